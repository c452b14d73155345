// Periodic (2D lattice) systems: Ewald parameter, the drop-in
// qpms_scatsyswk_build_modeproblem_matrix_full[_LU], and the batched
// dispersion scan (assembly over (omega, Bloch vector) -> LU -> log|det| ->
// plane-wave excitation).
#include <cublas_v2.h>
#include <math.h>
#include <stddef.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "qg_assembly.h"
#include "qg_batched.h"
#include "qg_ewald.h"
#include "qg_internal.h"
#include "qg_specfunc.cuh"

namespace qg {
bool scatsys_is_own(const qpms_scatsys_t *ss);
int scatsys_lmax(const qpms_scatsys_t *ss);
void scatsys_tdiag(const qpms_scatsys_t *ss, int t, double om_re, double om_im, std::vector<qg_c> &out);
qg_c scatsys_wavenumber(const qpms_scatsys_t *ss, double om_re, double om_im);
void planewave_direction_coeffs(int lMax, const double k_dir[3], const qpms_complex_t E_cart[3],
                                std::vector<qg_c> &coef);
int blas_handle_get(cublasHandle_t *h);
bool scatsys_dense(const qpms_scatsys_t *ss);

namespace {

struct Dev {
  void *p = nullptr;
  ~Dev() {
    if (p) cudaFree(p);
  }
  template <typename T>
  T *as() const {
    return reinterpret_cast<T *>(p);
  }
};
int dalloc(Dev &b, size_t bytes) {
  QG_CUDA_TRY(cudaMalloc(&b.p, bytes ? bytes : 16));
  return QPMS_SUCCESS;
}

double fact(int n) {
  double f = 1;
  for (int i = 2; i <= n; ++i) f *= i;
  return f;
}

// Lattice constants of the Ewald kernel (ewald.c:104-157, 228-241).
int build_ewald_const(const qpms_scatsys_t *ss, int lMax, EwaldConst *c, int csphase = -1) {
  const int LE = 2 * lMax + 1;
  if (LE > kEwLE) {
    set_error("periodic systems support lMax <= %d", (kEwLE - 1) / 2);
    return QPMS_EINVAL;
  }
  memset(c, 0, sizeof *c);
  const cart3_t b1 = ss->per.lattice_basis[0], b2 = ss->per.lattice_basis[1];
  c->b[0] = b1.x; c->b[1] = b1.y; c->b[2] = b2.x; c->b[3] = b2.y;
  const double det = b1.x * b2.y - b1.y * b2.x;
  c->rb[0] = 2 * M_PI * b2.y / det;
  c->rb[1] = -2 * M_PI * b2.x / det;
  c->rb[2] = -2 * M_PI * b1.y / det;
  c->rb[3] = 2 * M_PI * b1.x / det;
  c->bn[0] = hypot(c->b[0], c->b[1]);
  c->bn[1] = hypot(c->b[2], c->b[3]);
  c->rbn[0] = hypot(c->rb[0], c->rb[1]);
  c->rbn[1] = hypot(c->rb[2], c->rb[3]);
  c->area = fabs(det);
  std::vector<double> P((LE + 1) * (LE + 2) / 2);
  for (int m = 0; m <= LE; ++m) legendre_column(LE, m, 0.0, P.data());  // csphase -1 (default normalisation)
  int off = 0;
  for (int n = 0; n <= LE; ++n)
    for (int m = -n; m <= n; ++m) {
      const int y = n * (n + 1) + m, am = m < 0 ? -m : m;
      const double sgn = (m < 0 && (m % 2)) ? -1.0 : 1.0;
      // legendre_column carries the Condon-Shortley phase (-1)^m; csphase +1 drops it
      const double cs = (csphase == -1 || (am % 2) == 0) ? 1.0 : -1.0;
      c->leg0m[y] = P[n * (n + 1) / 2 + am] * sgn * cs;
      c->s1off[y] = off;
      if ((m + n) % 2 == 0) {
        static const double ipr[4][2] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}};
        const double *ip = ipr[(n + 1) % 4];
        for (int j = 0; j <= (n - am) / 2; ++j) {
          const double f = -2 * 1.7724538509055160273 * fact((n - m) / 2) * fact((n + m) / 2) * ((j % 2) ? -1 : 1) /
                           (fact(j) * fact((n - m) / 2 - j) * fact((n + m) / 2 - j)) * c->leg0m[y];
          c->s1[off + j] = cmk(f * ip[0], f * ip[1]);
          c->s1r[off + j] = f;
        }
        off += (n - am) / 2 + 1;
      }
    }
  // shifted layers: leg_nm sign factors and the S1[y][j, s] constants
  //   S1 = -i (-1)^n 2 sqrt(pi) L_nm (-i)^mu c_t (-1)^(t+s) H_{s, s-j} 2^-s
  // (mu = |m|, t = (n - mu - s) / 2, H_{s,l} = s! (-1)^l / (l! (s - 2l)!),
  // r^n P_n^mu(cos theta) = rho^mu sum_t c_t rho^(2t) z^(n - mu - 2t) without
  // the Condon-Shortley phase, L_nm = legs[y] (-1)^mu): the Gaussian-regularised
  // h_n Y_nm summed over the lattice by 2D Poisson summation, z derivatives as
  // Hermite polynomials.  At z = 0 only 2j = s remains and equals s1 above.
  int zo = 0;
  for (int n = 0; n <= LE; ++n)
    for (int m = -n; m <= n; ++m) {
      const int y = n * (n + 1) + m, mu = m < 0 ? -m : m, LM = n - mu;
      const double msgn = (m < 0 && (m % 2)) ? -1.0 : 1.0;
      c->legs[y] = msgn * ((csphase == -1 || (mu % 2) == 0) ? 1.0 : -1.0);
      const double L = c->legs[y] * ((mu % 2) ? -1.0 : 1.0);
      // -i (-1)^n (-i)^mu = (-i)^(mu + 1) (-1)^n
      static const double mi[4][2] = {{1, 0}, {0, -1}, {-1, 0}, {0, 1}};  // (-i)^p
      const double *ph = mi[(mu + 1) % 4];
      const double pre = ((n % 2) ? -1.0 : 1.0) * 2 * 1.7724538509055160273 * L;
      c->zoff[y] = zo;
      for (int j = 0; j <= LM; ++j)
        for (int sv = j + (LM - j) % 2; sv <= 2 * j && sv <= LM; sv += 2) {
          const int t = (LM - sv) / 2, l = sv - j;
          double ct = 0;
          for (int kk = t; kk <= LM / 2; ++kk)
            ct += ldexp(1.0, -n) * ((kk % 2) ? -1.0 : 1.0) * fact(n) / (fact(kk) * fact(n - kk)) *
                  fact(2 * n - 2 * kk) / (fact(n) * fact(n - 2 * kk)) * fact(n - 2 * kk) / fact(n - 2 * kk - mu) *
                  fact(kk) / (fact(t) * fact(kk - t));
          const double h = fact(sv) * ((l % 2) ? -1.0 : 1.0) / (fact(l) * fact(sv - 2 * l));
          const double v = pre * ct * (((t + sv) % 2) ? -1.0 : 1.0) * h * ldexp(1.0, -sv);
          if (zo >= kEwZ) {
            set_error("shifted Ewald constants: table overflow");
            return QPMS_ERROR;
          }
          c->zs1[zo] = cmk(v * ph[0], v * ph[1]);
          c->zj[zo] = (unsigned char)j;
          c->zsv[zo] = (unsigned char)sv;
          ++zo;
        }
    }
  c->zoff[(LE + 1) * (LE + 1)] = zo;
  return QPMS_SUCCESS;
}

// 1 if the np positions (x, y, z) do not all lie in one plane z = const:
// the Ewald assembly then also runs its kernel for pairs of layers.
int layered_positions(const double *pos, size_t np) {
  for (size_t i = 1; i < np; ++i)
    if (pos[3 * i + 2] != pos[2]) return 1;
  return 0;
}

}  // namespace

// layered_positions for the particles of ss
int layered_system(const qpms_scatsys_t *ss) {
  for (qpms_ss_pi_t i = 1; i < ss->p_count; ++i)
    if (ss->p[i].pos.z != ss->p[0].pos.z) return 1;
  return 0;
}

namespace {

// log|det| of nb row-major N x N LU factors (column-major getrf of M^T has
// the same diagonal of U)
__global__ void logdet_kernel(int nb, int N, const qg_c *LU, double *out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const qg_c *A = LU + (size_t)b * N * N;
  double s = 0;
  for (int i = 0; i < N; ++i) s += log(hypot(A[(size_t)i * N + i].re, A[(size_t)i * N + i].im));
  out[b] = s;
}

}  // namespace

// The lattice constants live in __constant__ memory, one lattice at a time:
// every Ewald assembly (any thread, any stream) holds this lock from the
// constant upload until its kernel has finished.
std::mutex &ewald_mutex() {
  static std::mutex m;
  return m;
}

// Upload the lattice constants of ss and run the Ewald assembly described by
// a (device buffers filled by the caller, *a.err zeroed here) on stream st;
// returns after the kernel has finished.
int ewald_assemble_locked(const qpms_scatsys_t *ss, const EwaldArgs &a, cudaStream_t st) {
  EwaldConst ec;
  int e;
  const int csphase = (ss->c->normalisation & QPMS_NORMALISATION_CSPHASE) ? -1 : 1;
  if ((e = build_ewald_const(ss, ss->c->lMax, &ec, csphase))) return e;
  std::lock_guard<std::mutex> lk(ewald_mutex());
  QG_CUDA_TRY(cudaMemsetAsync(a.err, 0, 4, st));
  if ((e = ewald_upload_constants(ec, st))) return e;
  if ((e = launch_ewald_assemble(a, priv(ss->c)->dev, st))) return e;
  int herr = 0;
  QG_CUDA_TRY(cudaMemcpyAsync(&herr, a.err, 4, cudaMemcpyDeviceToHost, st));
  QG_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr & 2) {
    set_error("Ewald sum: pair of layers at different heights without the layered flag");
    return QPMS_ERROR;
  }
  if (herr) {
    set_error("Ewald sum: lattice-point range above the bound (wavenumber or eta out of range)");
    return QPMS_ERROR;
  }
  return QPMS_SUCCESS;
}

namespace {
// Pointer arrays of the batched GEMM C_R = -T_R X_R (one entry per (matrix,
// particle)): X_R,: is rows [R n, R n + n) of the row-major N x N matrix X,
// i.e. the column-major N x n matrix X_R^T (ld N); T_R row-major is the
// column-major T_R^T (ld n); C_R^T = X_R^T T_R^T.
__global__ void dense_t_ptrs_kernel(int nmat, int np, int n, int N, int ntm, int nk, int paired,
                                    const int *__restrict__ tmid, const qg_c *X, const qg_c *T, qg_c *M,
                                    const void **pa, const void **pb, void **pc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nmat * np) return;
  const int m = i / np, R = i % np, w = paired ? m : m / nk;
  const size_t off = (size_t)m * N * N + (size_t)R * n * N;
  pa[i] = X + off;
  pb[i] = T + ((size_t)w * ntm + tmid[R]) * n * n;
  pc[i] = M + off;
}

// M (already -T_R X_R,:) += I + T_R on the diagonal blocks.
__global__ void dense_t_diag_kernel(int nmat, int np, int n, int N, int ntm, int nk, int paired,
                                    const int *__restrict__ tmid, const qg_c *__restrict__ T, qg_c *M) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nn = (size_t)n * n;
  if (i >= (size_t)nmat * np * nn) return;
  const int m = (int)(i / ((size_t)np * nn));
  const int R = (int)((i / nn) % np);
  const int a = (int)((i % nn) / n), b = (int)(i % n);
  const int w = paired ? m : m / nk;
  qg_c t = T[((size_t)w * ntm + tmid[R]) * nn + (size_t)a * n + b];
  if (a == b) t.re += 1.0;
  qg_c &o = M[(size_t)m * N * N + (size_t)(R * n + a) * N + R * n + b];
  o = cadd(o, t);
}
}  // namespace

// The lattice assembly for dense T-matrices (a.T: [nw][ntm][n][n] row-major):
// the Ewald kernel scales rows by a diagonal T, so it builds X = I + W with
// T = -1 first; then M_R,: = (I + T_R) delta_R,: - T_R X_R,: by one batched
// complex GEMM per (matrix, particle) block row and a diagonal-block kernel.
int ewald_assemble_dense(const qpms_scatsys_t *ss, const EwaldArgs &a, int n, cudaStream_t st) {
  const int np = a.np, N = np * n;
  const int nmat = a.paired ? a.nw : a.nw * a.nk;
  const size_t NN = (size_t)N * N, nb = (size_t)nmat * np;
  void *buf = nullptr;
  const size_t bx = (size_t)nmat * NN * 16, bm = ((size_t)a.nw * a.ntm * n * 16 + 255) / 256 * 256,
               bp = 3 * nb * sizeof(void *);
  QG_CUDA_TRY(cudaMallocAsync(&buf, bx + bm + bp, st));
  qg_c *X = (qg_c *)buf;
  qg_c *Tm1 = (qg_c *)((char *)buf + bx);
  void **ptrs = (void **)((char *)buf + bx + bm);
  int e = QPMS_SUCCESS;
  {
    std::vector<qg_c> m1((size_t)a.nw * a.ntm * n, cmk(-1.0, 0.0));
    cudaError_t ce = cudaMemcpyAsync(Tm1, m1.data(), m1.size() * 16, cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);  // m1 is a local buffer
    if (ce != cudaSuccess) {
      cudaFreeAsync(buf, st);
      QG_CUDA_TRY(ce);
    }
  }
  EwaldArgs ax = a;
  ax.T = Tm1;
  ax.M = X;
  e = ewald_assemble_locked(ss, ax, st);
  cublasHandle_t h;
  if (!e) e = blas_handle_get(&h);
  if (!e) {
    dense_t_ptrs_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(
        nmat, np, n, N, a.ntm, a.nk, a.paired, a.tmid, X, a.T, a.M, (const void **)ptrs, (const void **)(ptrs + nb),
        ptrs + 2 * nb);
    g_launches.fetch_add(1);
    const cuDoubleComplex mone = make_cuDoubleComplex(-1, 0), zero = make_cuDoubleComplex(0, 0);
    if (cudaGetLastError() != cudaSuccess || cublasSetStream(h, st) != CUBLAS_STATUS_SUCCESS ||
        cublasZgemmBatched(h, CUBLAS_OP_N, CUBLAS_OP_N, N, n, n, &mone, (const cuDoubleComplex **)ptrs, N,
                           (const cuDoubleComplex **)(ptrs + nb), n, &zero, (cuDoubleComplex **)(ptrs + 2 * nb), N,
                           (int)nb) != CUBLAS_STATUS_SUCCESS) {
      set_error("dense T: batched GEMM failed");
      e = QPMS_ERROR;
    } else {
      g_launches.fetch_add(1);
      const size_t tot = nb * n * n;
      dense_t_diag_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(nmat, np, n, N, a.ntm, a.nk, a.paired,
                                                                         a.tmid, a.T, a.M);
      g_launches.fetch_add(1);
      if (cudaGetLastError() != cudaSuccess) { set_error("dense T: diagonal-block kernel failed"); e = QPMS_ERROR; }
    }
  }
  cudaFreeAsync(buf, st);
  return e;
}

// Batched periodic assembly into device memory: nw frequencies x nk Bloch vectors.
int periodic_assemble_device_ex(const qpms_scatsys_t *ss, int nw, const qg_c *k_host,
                                const std::vector<qg_c> &T_host, int nk, const double *beta_host,
                                const double *eta_host, qg_c *dM, cudaStream_t st, bool sr_tables);

int periodic_assemble_device(const qpms_scatsys_t *ss, int nw, const qg_c *k_host,
                                    const std::vector<qg_c> &T_host, int nk, const double *beta_host,
                                    const double *eta_host, qg_c *dM, cudaStream_t st) {
  return periodic_assemble_device_ex(ss, nw, k_host, T_host, nk, beta_host, eta_host, dM, st, false);
}

// sr_tables: eta_host is one value per frequency (eta_host[w * nk + k] the
// same for every k); the short-range terms are then formed once per
// (frequency, particle pair) and shared by the nk Bloch vectors.
int periodic_assemble_device_ex(const qpms_scatsys_t *ss, int nw, const qg_c *k_host,
                                const std::vector<qg_c> &T_host, int nk, const double *beta_host,
                                const double *eta_host, qg_c *dM, cudaStream_t st, bool sr_tables) {
  const int np = ss->p_count;
  int e;
  std::vector<double> pos(3 * np);
  std::vector<int> tm(np);
  for (int i = 0; i < np; ++i) {
    pos[3 * i] = ss->p[i].pos.x;
    pos[3 * i + 1] = ss->p[i].pos.y;
    pos[3 * i + 2] = ss->p[i].pos.z;
    tm[i] = ss->p[i].tmatrix_id;
  }
  // the Ewald parameter sets how many lattice points each sum visits
  for (size_t i = 0; i < (size_t)nw * nk; ++i)
    if (!(eta_host[i] >= 0.05 * ss->per.eta && eta_host[i] <= 50 * ss->per.eta)) {
      set_error("Ewald eta %g outside [0.05, 50] x the lattice default %g", eta_host[i], ss->per.eta);
      return QPMS_EINVAL;
    }
  Dev dpos, dtm, dT, dk, dbeta, deta, derr;
  if ((e = dalloc(derr, 4))) return e;
  if ((e = dalloc(dpos, pos.size() * 8)) || (e = dalloc(dtm, np * 4)) || (e = dalloc(dT, T_host.size() * 16)) ||
      (e = dalloc(dk, nw * 16)) || (e = dalloc(dbeta, nk * 16)) || (e = dalloc(deta, (size_t)nw * nk * 8)))
    return e;
  QG_CUDA_TRY(cudaMemcpyAsync(dpos.p, pos.data(), pos.size() * 8, cudaMemcpyHostToDevice, st));
  QG_CUDA_TRY(cudaMemcpyAsync(dtm.p, tm.data(), np * 4, cudaMemcpyHostToDevice, st));
  QG_CUDA_TRY(cudaMemcpyAsync(dT.p, T_host.data(), T_host.size() * 16, cudaMemcpyHostToDevice, st));
  QG_CUDA_TRY(cudaMemcpyAsync(dk.p, k_host, nw * 16, cudaMemcpyHostToDevice, st));
  QG_CUDA_TRY(cudaMemcpyAsync(dbeta.p, beta_host, nk * 16, cudaMemcpyHostToDevice, st));
  QG_CUDA_TRY(cudaMemcpyAsync(deta.p, eta_host, (size_t)nw * nk * 8, cudaMemcpyHostToDevice, st));
  EwaldArgs a;
  a.nw = nw;
  a.nk = nk;
  a.np = np;
  a.ntm = ss->tm_count;
  a.pos = dpos.as<double>();
  a.tmid = dtm.as<int>();
  a.T = dT.as<qg_c>();
  a.k = dk.as<qg_c>();
  a.beta = dbeta.as<double>();
  a.eta = deta.as<double>();
  a.M = dM;
  a.err = derr.as<int>();
  a.layered = layered_positions(pos.data(), np);
  Dev dtab, dpts, dcnt;
  if (sr_tables) {
    for (int w = 0; w < nw; ++w)
      for (int k = 1; k < nk; ++k)
        if (eta_host[(size_t)w * nk + k] != eta_host[(size_t)w * nk]) {
          set_error("internal: short-range tables need one eta per frequency");
          return QPMS_ERROR;
        }
    // table size: the lattice-index box of the short-range sum at the
    // smallest eta (same bound as the kernels: |R - s| eta <= 7.5)
    double emin = eta_host[0];
    for (int w = 0; w < nw; ++w) emin = std::min(emin, eta_host[(size_t)w * nk]);
    const double rbn0 = hypot(ss->per.reciprocal_basis[0].x, ss->per.reciprocal_basis[0].y);
    const double rbn1 = hypot(ss->per.reciprocal_basis[1].x, ss->per.reciprocal_basis[1].y);
    long srmax = 1;
    for (int R = 0; R < np; ++R)
      for (int C = 0; C < np; ++C) {
        const double smax = hypot(pos[3 * R] - pos[3 * C], pos[3 * R + 1] - pos[3 * C + 1]);
        const long I1 = (long)ceil((7.5 / emin + smax) * rbn0) + 1, I2 = (long)ceil((7.5 / emin + smax) * rbn1) + 1;
        srmax = std::max(srmax, (2 * I1 + 1) * (2 * I2 + 1));
      }
    const int lMax = scatsys_lmax(ss), LE = 2 * lMax + 1, nev = (LE + 1) * (LE + 2) / 2;
    const size_t units = (size_t)nw * np * np;
    if ((e = dalloc(dtab, units * nev * srmax * 16)) || (e = dalloc(dpts, units * srmax * 16)) ||
        (e = dalloc(dcnt, units * 4)))
      return e;
    a.srtab = dtab.as<qg_c>();
    a.srpts = dpts.as<double>();
    a.srcnt = dcnt.as<int>();
    a.srmax = (int)srmax;
  }
  const int n = (int)(ss->fecv_size / np);
  if (T_host.size() == (size_t)nw * ss->tm_count * n * n && n > 1) return ewald_assemble_dense(ss, a, n, st);
  return ewald_assemble_locked(ss, a, st);
}

}  // namespace qg

using namespace qg;

namespace qg {
namespace {
// Field of a 2D-periodic array at points from the lattice-summed
// blocks W(point <- particle) (pair-list Ewald assembly with T = -1, so a
// block is W itself): a = sum_p W_qp f_p, of which only the electric l = 1
// regular waves are non-zero at the point itself; E = sum_m a_(N,1,m) D_m with
// D_m the cartesian value of the regular electric dipole wave at r = 0.
// One block per point, deterministic reduction order.
__global__ void periodic_field_kernel(int npts, int np, int n, const qg_c *__restrict__ W,
                                      const qg_c *__restrict__ f, const qg_c *__restrict__ D,
                                      qg_c *__restrict__ E) {
  const int q = blockIdx.x;
  if (q >= npts) return;
  __shared__ qg_c red[3][128];
  qg_c acc[3] = {cmk(0, 0), cmk(0, 0), cmk(0, 0)};
  const int tot = np * n;
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    const int p = t / n, c = t - p * n;
    const qg_c fc = f[(size_t)p * n + c];
    const qg_c *Wb = W + ((size_t)q * np + p) * n * n;
#pragma unroll
    for (int j = 0; j < 3; ++j) acc[j] = cadd(acc[j], cmul(Wb[(size_t)j * n + c], fc));
  }
  for (int j = 0; j < 3; ++j) red[j][threadIdx.x] = acc[j];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int j = 0; j < 3; ++j) red[j][threadIdx.x] = cadd(red[j][threadIdx.x], red[j][threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x < 3) {
    const int x = threadIdx.x;
    qg_c e = cmk(0, 0);
    for (int j = 0; j < 3; ++j) e = cadd(e, cmul(red[j][0], D[3 * j + x]));
    E[(size_t)q * 3 + x] = e;
  }
}
}  // namespace

// Regular electric dipole waves N_(1,m), m = -1, 0, 1, at r = 0 in cartesian
// components, default normalisation (qpms_vswf_fill_csph at kr = 0: besfac
// 1/3, besderfac 2/3, evaluated at theta = pi/2, phi = 0 as
// scatsystem.c:2118-2124 does): D[3 m' + x].
void regular_dipoles_at_origin(qg_c *D) {
  const double leg1 = -sqrt(3.0 / (16 * M_PI));          // leg(1, 1) = pi(1, +-1)
  const double tau0 = -sqrt(3.0 / (4 * M_PI)) / sqrt(2.0);  // tau(1, 0)
  // (r, theta, phi) components -> cartesian at theta = pi/2, phi = 0: x = r, y = phi, z = -theta
  const qg_c Nm1[3] = {cmk(-2.0 / 3 * leg1, 0), cmk(0, 2.0 / 3 * leg1), cmk(0, 0)};
  const qg_c N0[3] = {cmk(0, 0), cmk(0, 0), cmk(-2.0 / 3 * tau0, 0)};
  const qg_c Np1[3] = {cmk(2.0 / 3 * leg1, 0), cmk(0, 2.0 / 3 * leg1), cmk(0, 0)};
  for (int x = 0; x < 3; ++x) {
    D[x] = Nm1[x];
    D[3 + x] = N0[x];
    D[6 + x] = Np1[x];
  }
}

// E at npts points (host where / E), lattice sums at (k, beta, eta); points
// off the particles' plane use the sums for layers at different heights.
int periodic_field(const qpms_scatsys_t *ss, qg_c k, const double beta[2], double eta, const qg_c *cvf_host,
                   size_t npts, const double *where, qg_c *E_host) {
  const int np = ss->p_count;
  const int n = (int)(ss->fecv_size / np);
  if (!(eta >= 0.05 * ss->per.eta && eta <= 50 * ss->per.eta)) {
    set_error("Ewald eta %g outside [0.05, 50] x the lattice default %g", eta, ss->per.eta);
    return QPMS_EINVAL;
  }
  if (npts == 0) return QPMS_SUCCESS;
  // points per chunk: the W blocks of a chunk stay below 256 MiB
  const size_t per_pt = (size_t)np * n * n * 16;
  const size_t chunk = std::max<size_t>(1, std::min<size_t>(npts, ((size_t)256 << 20) / per_pt));
  qg_c D[9];
  regular_dipoles_at_origin(D);
  std::vector<qg_c> Tm1(n, cmk(-1.0, 0.0));
  Dev dpos, dtm, dT, dk, dbeta, deta, derr, dpairs, dW, df, dD, dE;
  int e;
  if ((e = dalloc(dpos, (np + chunk) * 24)) || (e = dalloc(dtm, (np + chunk) * 4)) || (e = dalloc(dT, n * 16)) ||
      (e = dalloc(dk, 16)) || (e = dalloc(dbeta, 16)) || (e = dalloc(deta, 8)) || (e = dalloc(derr, 4)) ||
      (e = dalloc(dpairs, chunk * np * 8)) || (e = dalloc(dW, chunk * per_pt)) ||
      (e = dalloc(df, ss->fecv_size * 16)) || (e = dalloc(dD, 9 * 16)) || (e = dalloc(dE, chunk * 48)))
    return e;
  std::vector<int> tm(np + chunk, 0), pairs(2 * chunk * np);
  QG_CUDA_TRY(cudaMemcpy(dtm.p, tm.data(), tm.size() * 4, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dT.p, Tm1.data(), n * 16, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dk.p, &k, 16, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dbeta.p, beta, 16, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(deta.p, &eta, 8, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(df.p, cvf_host, ss->fecv_size * 16, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dD.p, D, 9 * 16, cudaMemcpyHostToDevice));
  std::vector<double> pos(3 * (np + chunk));
  for (int i = 0; i < np; ++i) {
    pos[3 * i] = ss->p[i].pos.x;
    pos[3 * i + 1] = ss->p[i].pos.y;
    pos[3 * i + 2] = ss->p[i].pos.z;
  }
  for (size_t q0 = 0; q0 < npts; q0 += chunk) {
    const size_t m = std::min(chunk, npts - q0);
    memcpy(&pos[3 * np], where + 3 * q0, m * 24);
    for (size_t q = 0; q < m; ++q)
      for (int p = 0; p < np; ++p) {
        pairs[2 * (q * np + p)] = (int)(np + q);  // destination: the point
        pairs[2 * (q * np + p) + 1] = p;          // source: particle p
      }
    QG_CUDA_TRY(cudaMemcpy(dpos.p, pos.data(), (np + m) * 24, cudaMemcpyHostToDevice));
    QG_CUDA_TRY(cudaMemcpy(dpairs.p, pairs.data(), m * np * 8, cudaMemcpyHostToDevice));
    EwaldArgs a;
    a.nw = 1;
    a.nk = 1;
    a.np = (int)(np + m);
    a.ntm = 1;
    a.pos = dpos.as<double>();
    a.tmid = dtm.as<int>();
    a.T = dT.as<qg_c>();
    a.k = dk.as<qg_c>();
    a.beta = dbeta.as<double>();
    a.eta = deta.as<double>();
    a.M = dW.as<qg_c>();
    a.err = derr.as<int>();
    a.npairs = (int)(m * np);
    a.pairs = dpairs.as<int>();
    a.layered = layered_positions(pos.data(), np + m);
    if ((e = ewald_assemble_locked(ss, a, 0))) return e;
    periodic_field_kernel<<<(unsigned)m, 128>>>((int)m, np, n, dW.as<qg_c>(), df.as<qg_c>(), dD.as<qg_c>(),
                                                dE.as<qg_c>());
    g_launches.fetch_add(1);
    QG_CUDA_TRY(cudaGetLastError());
    QG_CUDA_TRY(cudaMemcpy(E_host + 3 * q0, dE.p, m * 48, cudaMemcpyDeviceToHost));
  }
  return QPMS_SUCCESS;
}
}  // namespace qg

extern "C" {

double qpms_ss_adjusted_eta(const qpms_scatsys_t *ss, qpms_complex_t wavenumber, const double wavevector[3]) {
  // scatsystem.c:68-80
  const double eta_default = ss->per.eta;
  const double k2 = wavevector[0] * wavevector[0] + wavevector[1] * wavevector[1] + wavevector[2] * wavevector[2];
  const double kappa2 = wavenumber.re * wavenumber.re + wavenumber.im * wavenumber.im;
  if (kappa2 < k2) return eta_default;
  const int maxj = ss->c->lMax;
  const double mina = 0.5 * (ss->lattice_dimension - 1) - maxj;
  const double eta_min = sqrt(fabs((kappa2 - k2) * (mina - 1.) / 16.));
  return std::max(eta_default, eta_min);
}

qpms_complex_t *qpms_scatsyswk_build_modeproblem_matrix_full(qpms_complex_t *target,
                                                             const qpms_scatsys_at_omega_k_t *sswk) {
  clear_error();
  if (!sswk || !sswk->ssw) { set_error("NULL sswk"); return nullptr; }
  const qpms_scatsys_at_omega_t *ssw = sswk->ssw;
  const qpms_scatsys_t *ss = ssw->ss;
  if (ss->lattice_dimension != 2) { set_error("only 2D lattices are supported"); return nullptr; }
  if (sswk->k[2] != 0) { set_error("Bloch vector must lie in the xy plane"); return nullptr; }
  const size_t N = ss->fecv_size, n = ssw->tm[0]->spec->n;
  std::vector<qg_c> T;
  bool diag = true;
  for (int t = 0; t < ss->tm_count; ++t)
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < n; ++j)
        if (i != j && (ssw->tm[t]->m[i * n + j].re != 0 || ssw->tm[t]->m[i * n + j].im != 0)) diag = false;
  for (int t = 0; t < ss->tm_count; ++t)
    for (size_t i = 0; i < n; ++i) {
      if (!diag) {  // dense T-matrices: the GEMM path of the lattice assembly
        for (size_t j = 0; j < n; ++j) T.push_back(*(const qg_c *)&ssw->tm[t]->m[i * n + j]);
        continue;
      }
      T.push_back(*(const qg_c *)&ssw->tm[t]->m[i * n + i]);
    }
  const qg_c k = *(const qg_c *)&ssw->wavenumber;
  double eta = sswk->eta;
  if (eta == 0 || isnan(eta)) eta = qpms_ss_adjusted_eta(ss, ssw->wavenumber, sswk->k);
  const double beta[2] = {sswk->k[0], sswk->k[1]};
  Dev dM;
  if (dalloc(dM, N * N * 16)) return nullptr;
  if (periodic_assemble_device(ss, 1, &k, T, 1, beta, &eta, dM.as<qg_c>(), 0)) return nullptr;
  bool own = false;
  if (!target) {
    target = (qpms_complex_t *)malloc(N * N * 16);
    own = true;
  }
  if (cudaMemcpy(target, dM.p, N * N * 16, cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("device to host copy failed");
    if (own) free(target);
    return nullptr;
  }
  return target;
}

qpms_ss_LU qpms_scatsyswk_build_modeproblem_matrix_full_LU(qpms_complex_t *target, int *target_piv,
                                                           const qpms_scatsys_at_omega_k_t *sswk) {
  qpms_complex_t *M = qpms_scatsyswk_build_modeproblem_matrix_full(target, sswk);
  if (!M) {
    qpms_ss_LU lu;
    memset(&lu, 0, sizeof lu);
    return lu;
  }
  return qpms_scatsysw_modeproblem_matrix_full_factorise(M, target_piv, sswk->ssw, sswk);
}

int qpms_gpu_periodic_scan(const qpms_scatsys_t *ss, size_t nw, const double *omegas, size_t nk,
                           const double *kvecs, int mode, double *logdet, qpms_complex_t *f_out, double *sigma_ext,
                           double *resid_out, int *iters_out) {
  clear_error();
  if (!scatsys_is_own(ss) || ss->lattice_dimension != 2) {
    set_error("system must come from qpms_gpu_scatsys_create_spheres_2d");
    return QPMS_EINVAL;
  }
  if (!omegas || !kvecs || !logdet) { set_error("NULL argument"); return QPMS_EINVAL; }
  if (mode != 0 && mode != 1) { set_error("mode must be 0 (FP64) or 1 (mixed)"); return QPMS_EINVAL; }
  if (!nw || !nk) return QPMS_SUCCESS;
  const int lMax = scatsys_lmax(ss), np = ss->p_count, ntm = ss->tm_count, n = 2 * lMax * (lMax + 2);
  const size_t N = ss->fecv_size, N2 = N * N;
  cublasHandle_t h;
  int e;
  if ((e = blas_handle_get(&h))) return e;
  // process in chunks of whole frequencies, <= ~2 GiB of matrices per chunk
  const size_t per_w = nk * N2 * 16;
  const int wchunk = (int)std::max<size_t>(1, std::min<size_t>(nw, (size_t(2) << 30) / per_w));
  std::vector<double> pos(3 * np);
  std::vector<int> tm(np);
  for (int i = 0; i < np; ++i) {
    pos[3 * i] = ss->p[i].pos.x;
    pos[3 * i + 1] = ss->p[i].pos.y;
    pos[3 * i + 2] = ss->p[i].pos.z;
    tm[i] = ss->p[i].tmatrix_id;
  }
  Dev dM, dscr, dlog, dT, dtm, dpos, dk, dkv, dcf, da, db, dx, dsig;
  const size_t nmat = (size_t)wchunk * nk;
  if ((e = dalloc(dM, nmat * N2 * 16)) || (e = dalloc(dscr, batched_solve_bytes((int)nmat, N, mode))) ||
      (e = dalloc(dlog, nmat * 8)) || (e = dalloc(dtm, np * 4)) || (e = dalloc(dpos, np * 24)) ||
      (e = dalloc(da, nmat * N * 16)) || (e = dalloc(db, nmat * N * 16)) || (e = dalloc(dx, nmat * N * 16)) ||
      (e = dalloc(dsig, nmat * 8)) || (e = dalloc(dk, nmat * 16)) || (e = dalloc(dkv, nmat * 24)) ||
      (e = dalloc(dT, nmat * ntm * (scatsys_dense(ss) ? (size_t)n * n : n) * 16)) ||
      (e = dalloc(dcf, nmat * n * 16)))
    return e;
  QG_CUDA_TRY(cudaMemcpy(dtm.p, tm.data(), np * 4, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dpos.p, pos.data(), np * 24, cudaMemcpyHostToDevice));
  std::vector<double> res(nmat);
  std::vector<int> its(nmat), info(nmat);
  for (size_t w0 = 0; w0 < nw; w0 += wchunk) {
    const int W = (int)std::min<size_t>(wchunk, nw - w0);
    const size_t nm = (size_t)W * nk;
    std::vector<qg_c> T, k(W), kk(nm), Tm;
    std::vector<double> eta(nm), kvec(3 * nm);
    std::vector<qg_c> coefs(nm * n);
    for (int w = 0; w < W; ++w) {
      for (int t = 0; t < ntm; ++t) {
        std::vector<qg_c> d;
        scatsys_tdiag(ss, t, omegas[w0 + w], 0.0, d);
        T.insert(T.end(), d.begin(), d.end());
      }
      k[w] = scatsys_wavenumber(ss, omegas[w0 + w], 0.0);
      const double kap = k[w].re;
      // one eta per frequency, the largest adjusted eta of its Bloch vectors
      // (the sums do not depend on eta; a larger one only moves work to the
      // long-range sum), so the short-range terms are shared by all of them
      double eta_w = 0;
      for (size_t ik = 0; ik < nk; ++ik) {
        const double kv[3] = {kvecs[2 * ik], kvecs[2 * ik + 1], 0.0};
        eta_w = std::max(eta_w, qpms_ss_adjusted_eta(ss, *(const qpms_complex_t *)&k[w], kv));
      }
      for (size_t ik = 0; ik < nk; ++ik) {
        const size_t m = (size_t)w * nk + ik;
        const double kv[3] = {kvecs[2 * ik], kvecs[2 * ik + 1], 0.0};
        eta[m] = eta_w;
        kk[m] = k[w];
        // incident plane wave with in-plane wavevector beta, E along x projected
        // perpendicular to k (x-polarised at normal incidence)
        const double b2 = kv[0] * kv[0] + kv[1] * kv[1];
        const double kz = kap * kap > b2 ? sqrt(kap * kap - b2) : 0.0;
        const double kd[3] = {kv[0], kv[1], kz};
        const double kn = sqrt(b2 + kz * kz);
        double E[3] = {1, 0, 0};
        const double ex = kd[0] / kn;
        for (int c = 0; c < 3; ++c) E[c] -= ex * kd[c] / kn;
        const double En = sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
        qpms_complex_t Ec[3];
        for (int c = 0; c < 3; ++c) Ec[c] = {E[c] / En, 0.0};
        std::vector<qg_c> cf;
        planewave_direction_coeffs(lMax, kd, Ec, cf);
        const bool prop = kap * kap > b2;
        for (int i = 0; i < n; ++i) coefs[m * n + i] = prop ? cf[i] : cmk(0, 0);
        for (int c = 0; c < 3; ++c) kvec[3 * m + c] = kd[c];
        const size_t tsz = scatsys_dense(ss) ? (size_t)n * n : (size_t)n;
        for (int t = 0; t < ntm; ++t) Tm.insert(Tm.end(), T.begin() + ((size_t)w * ntm + t) * tsz,
                                                T.begin() + ((size_t)w * ntm + t + 1) * tsz);
      }
    }
    if ((e = periodic_assemble_device_ex(ss, W, k.data(), T, (int)nk, kvecs, eta.data(), dM.as<qg_c>(), 0, true)))
      return e;
    // per-matrix incidence (coefficients and phases differ per (w, k)), b = T a
    QG_CUDA_TRY(cudaMemcpy(dcf.p, coefs.data(), coefs.size() * 16, cudaMemcpyHostToDevice));
    QG_CUDA_TRY(cudaMemcpy(dkv.p, kvec.data(), nm * 24, cudaMemcpyHostToDevice));
    QG_CUDA_TRY(cudaMemcpy(dk.p, kk.data(), nm * 16, cudaMemcpyHostToDevice));
    QG_CUDA_TRY(cudaMemcpy(dT.p, Tm.data(), Tm.size() * 16, cudaMemcpyHostToDevice));
    if ((e = launch_incident((int)nm, np, n, dcf.as<qg_c>(), dkv.as<double>(), dpos.as<double>(), da.as<qg_c>(), 0,
                             (size_t)n)))
      return e;
    if ((e = launch_apply_t((int)nm, np, n, ntm, scatsys_dense(ss) ? 1 : 0, dtm.as<int>(), dT.as<qg_c>(),
                            da.as<qg_c>(), db.as<qg_c>(), 0)))
      return e;
    // LU (complex128, or complex64 + FP64 refinement), log|det| from the factors
    if ((e = batched_solve(h, 0, (int)nm, N, dM.as<qg_c>(), db.as<qg_c>(), dx.as<qg_c>(), mode, 1e-13, 12, dscr.p,
                           res.data(), its.data(), info.data(), dlog.as<double>())))
      return e;
    QG_CUDA_TRY(cudaMemcpy(logdet + w0 * nk, dlog.p, nm * 8, cudaMemcpyDeviceToHost));
    if ((e = launch_sigma_ext((int)nm, N, da.as<qg_c>(), dx.as<qg_c>(), dk.as<qg_c>(), dsig.as<double>(), 0)))
      return e;
    if (sigma_ext) QG_CUDA_TRY(cudaMemcpy(sigma_ext + w0 * nk, dsig.p, nm * 8, cudaMemcpyDeviceToHost));
    if (f_out) QG_CUDA_TRY(cudaMemcpy(f_out + w0 * nk * N, dx.p, nm * N * 16, cudaMemcpyDeviceToHost));
    for (size_t m = 0; m < nm; ++m) {
      if (resid_out) resid_out[w0 * nk + m] = res[m];
      if (iters_out) iters_out[w0 * nk + m] = its[m];
    }
  }
  return QPMS_SUCCESS;
}


namespace {
// ---- Lattice-point "web" of PGen_xyWeb (latticegens.c:449-568) ----
// The reference enumerates the points of a 2D lattice in layers: in the
// reduced basis (r1, r2) (lattices2d.c, l2d_reduceBasis), layer L holds the
// points i r1 + j r2 with |i| + |j| = L for a rectangular basis and
// max(|i|, |j|, |i + j|) = L otherwise; the layers 0 .. last are generated,
// last = floor(maxR / h) (one less when last h == maxR), h the in-circle
// radius of the unit hexagon (l2d_hexWebInCircleRadius).
struct LatticeWeb {
  double r1[2], r2[2];
  bool rect;
  long last;
};

double dot2(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1]; }

void reduce_basis(const double *b1in, const double *b2in, double *o1, double *o2) {
  double b1[2] = {b1in[0], b1in[1]}, b2[2] = {b2in[0], b2in[1]};
  double B1 = dot2(b1, b1);
  double mu = round(dot2(b1, b2) / B1);
  b2[0] -= mu * b1[0];
  b2[1] -= mu * b1[1];
  double B2 = dot2(b2, b2);
  for (int guard = 0; B2 < B1 && guard < 64; ++guard) {
    std::swap(b1[0], b2[0]);
    std::swap(b1[1], b2[1]);
    B1 = B2;
    mu = round(dot2(b1, b2) / B1);
    b2[0] -= mu * b1[0];
    b2[1] -= mu * b1[1];
    B2 = dot2(b2, b2);
  }
  o1[0] = b1[0]; o1[1] = b1[1];
  o2[0] = b2[0]; o2[1] = b2[1];
}

LatticeWeb lattice_web(const double *b1, const double *b2, double maxR) {
  LatticeWeb w;
  reduce_basis(b1, b2, w.r1, w.r2);
  const double B1 = dot2(w.r1, w.r1), B2 = dot2(w.r2, w.r2);
  const double d[2] = {w.r2[0] - w.r1[0], w.r2[1] - w.r1[1]};
  w.rect = dot2(d, d) - B1 - B2 <= 1e-13 * (B1 + B2);  // l2d_detectRightAngles, BASIS_RTOL
  // in-circle radius: the triangle (r1, r2, third side) with the third side
  // r2 - r1, or r2 + r1 when the basis is obtuse; height onto the third side
  double s3[2] = {d[0], d[1]}, s2[2] = {w.r2[0], w.r2[1]};
  if (dot2(d, d) - B1 - B2 > 0) {
    s3[0] = w.r2[0]; s3[1] = w.r2[1];
    s2[0] = w.r2[0] + w.r1[0]; s2[1] = w.r2[1] + w.r1[1];
  }
  const double e1 = sqrt(B1), e2 = sqrt(dot2(s2, s2)), e3 = sqrt(dot2(s3, s3)), p = 0.5 * (e1 + e2 + e3);
  const double h = 2 * sqrt(p * (p - e1) * (p - e2) * (p - e3)) / e3;
  w.last = (maxR > 0 && h > 0) ? (long)floor(maxR / h) : -1;
  if (w.last >= 0 && w.last * h >= maxR) --w.last;
  return w;
}

// 1 if every lattice point p with |p - c| <= rad lies in the generated layers.
bool web_covers(const LatticeWeb &w, double cx, double cy, double rad) {
  const double det = w.r1[0] * w.r2[1] - w.r1[1] * w.r2[0];
  if (det == 0 || !(rad >= 0)) return false;
  // |i| <= (|c| + rad) |r2| / |det| (distance between the lines i = const)
  const double reach = hypot(cx, cy) + rad;
  const long I = (long)ceil(reach * sqrt(dot2(w.r2, w.r2)) / fabs(det)) + 1;
  const long J = (long)ceil(reach * sqrt(dot2(w.r1, w.r1)) / fabs(det)) + 1;
  if (I > 4096 || J > 4096) return false;
  for (long i = -I; i <= I; ++i)
    for (long j = -J; j <= J; ++j) {
      const double px = i * w.r1[0] + j * w.r2[0] - cx, py = i * w.r1[1] + j * w.r2[1] - cy;
      if (px * px + py * py > rad * rad) continue;
      const long L = w.rect ? labs(i) + labs(j) : std::max(std::max(labs(i), labs(j)), labs(i + j));
      if (L > w.last) return false;
    }
  return true;
}
}  // namespace

// qpms_trans_calculator_get_AB_arrays_e32_e (translations.h:167-177,
// translations.c:926-1078): the lattice-summed A, B for one Bloch vector and
// particle shift.  Evaluated by the Ewald assembly kernel on a two-particle
// cell (positions shift and 0) with T = -1, whose off-diagonal block is then
// exactly W(shift) = [A B; B A].  Only the full sum is available (parts must
// be QPMS_EWALD_FULL).
//
// maxR / maxK: the reference sums the direct-lattice points R of the layers
// below maxR and the reciprocal points K of the layers below maxK
// (PGen_xyWeb, translations.c:960-1000).  The kernel's own cutoffs are set by
// the decay of the terms (|R - s| eta <= 7.5, x^2 <= 56).  When the caller's
// layers hold every point whose term is above ~1e-16 of the leading one
// (|R - s| eta <= 6, (|K + beta|^2 - |k|^2) / (4 eta^2) <= 36) the two sums
// agree to rounding; a maxR / maxK that cuts into that region asks for a
// truncated sum, which is not available: QPMS_EINVAL with a message.
//
// Aerr / Berr (if given): |A(eta) - A(1.25 eta)| elementwise (and the same
// for B), from a second evaluation in the same launch.  The full sum does not
// depend on eta, so the difference measures the truncation and rounding error
// of the evaluation (the reference propagates per-term quadrature and
// incomplete-gamma error estimates instead, ewald.c:420-468, 880-882).
int qpms_trans_calculator_get_AB_arrays_e32_e(const qpms_trans_calculator *c, qpms_complex_t *Adest, double *Aerr,
                                              qpms_complex_t *Bdest, double *Berr, ptrdiff_t deststride,
                                              ptrdiff_t srcstride, double eta, qpms_complex_t wavenumber,
                                              cart2_t b1, cart2_t b2, cart2_t beta, cart3_t particle_shift,
                                              double maxR, double maxK, int parts) {
  clear_error();
  if (!c || !Adest || !Bdest) { set_error("NULL argument"); return QPMS_EINVAL; }
  if (parts != 7) { set_error("only the full Ewald sum (QPMS_EWALD_FULL) is implemented"); return QPMS_EINVAL; }
  if (c->lMax > 4) { set_error("lattice sums need lMax <= 4"); return QPMS_EINVAL; }
  if (!(eta > 0)) { set_error("eta must be positive"); return QPMS_EINVAL; }
  const double bb1[2] = {b1.x, b1.y}, bb2[2] = {b2.x, b2.y};
  {
    if (fabs(bb1[0] * bb2[1] - bb1[1] * bb2[0]) <= 1e-13 * (dot2(bb1, bb1) + dot2(bb2, bb2))) {
      set_error("degenerate lattice basis");
      return QPMS_EINVAL;
    }
    const double z2 = particle_shift.z * particle_shift.z, rs = 6.0 / eta;
    const double rad_R = rs * rs > z2 ? sqrt(rs * rs - z2) : -1.0;
    const double det = bb1[0] * bb2[1] - bb1[1] * bb2[0];
    const double rk1[2] = {2 * M_PI * bb2[1] / det, -2 * M_PI * bb2[0] / det};
    const double rk2[2] = {-2 * M_PI * bb1[1] / det, 2 * M_PI * bb1[0] / det};
    const double k2 = wavenumber.re * wavenumber.re + wavenumber.im * wavenumber.im;
    const double rad_K = sqrt(k2 + 36.0 * 4 * eta * eta);
    const bool r_ok = rad_R < 0 || web_covers(lattice_web(bb1, bb2, maxR), particle_shift.x, particle_shift.y, rad_R);
    const bool k_ok = web_covers(lattice_web(rk1, rk2, maxK), -beta.x, -beta.y, rad_K);
    if (!r_ok || !k_ok) {
      set_error("%s truncates the lattice sum where its terms are above 1e-16 of the leading ones "
                "(needs %s >= about %.6g); truncated sums are not available",
                r_ok ? "maxK" : "maxR", r_ok ? "maxK" : "maxR",
                r_ok ? rad_K + hypot(beta.x, beta.y) : rad_R + hypot(particle_shift.x, particle_shift.y));
      return QPMS_EINVAL;
    }
  }
  const double pos[6] = {particle_shift.x, particle_shift.y, particle_shift.z, 0, 0, 0};
  const int kind[2] = {0, 0};
  const double rad = 1.0;
  qpms_complex_t eps_in, eps_med;
  eps_in.re = 2.0;
  eps_in.im = 0;
  eps_med.re = 1.0;
  eps_med.im = 0;
  qpms_scatsys_t *ss = qpms_gpu_scatsys_create_spheres_2d(2, pos, kind, 1, &rad, &eps_in, eps_med, c->lMax, bb1, bb2);
  if (!ss) return QPMS_ERROR;
  qpms_trans_calculator *own = ss->c;
  ss->c = const_cast<qpms_trans_calculator *>(c);  // the caller's normalisation and tables
  const int ne = c->nelem, n = 2 * ne, N = 2 * n;
  const bool doerr = Aerr || Berr;
  const int nk = doerr ? 2 : 1;  // (beta, eta) and, for the error estimate, (beta, 1.25 eta)
  std::vector<qg_c> T(n, cmk(-1.0, 0.0));
  const qg_c k = cmk(wavenumber.re, wavenumber.im);
  const double bt[4] = {beta.x, beta.y, beta.x, beta.y};
  const double etas[2] = {eta, 1.25 * eta};
  int e = QPMS_SUCCESS;
  std::vector<qg_c> M((size_t)nk * N * N);
  {
    Dev dM;
    if (!(e = dalloc(dM, M.size() * 16)))
      if (!(e = periodic_assemble_device(ss, 1, &k, T, nk, bt, etas, dM.as<qg_c>(), 0)))
        if (cudaMemcpy(M.data(), dM.p, M.size() * 16, cudaMemcpyDeviceToHost) != cudaSuccess) {
          set_error("device to host copy failed");
          e = QPMS_ERROR;
        }
  }
  ss->c = own;
  qpms_gpu_scatsys_free(ss);
  if (e) return e;
  // block (particle 0 <- particle 1): rows 0..n-1, columns n..2n-1
  const qg_c *M2 = M.data() + (size_t)(nk - 1) * N * N;
  for (int y = 0; y < ne; ++y)
    for (int yu = 0; yu < ne; ++yu) {
      const size_t ia = (size_t)y * N + n + yu, ib = ia + ne;
      const qg_c a = M[ia], b = M[ib];
      Adest[deststride * y + srcstride * yu].re = a.re;
      Adest[deststride * y + srcstride * yu].im = a.im;
      Bdest[deststride * y + srcstride * yu].re = b.re;
      Bdest[deststride * y + srcstride * yu].im = b.im;
      if (Aerr) Aerr[deststride * y + srcstride * yu] = hypot(a.re - M2[ia].re, a.im - M2[ia].im);
      if (Berr) Berr[deststride * y + srcstride * yu] = hypot(b.re - M2[ib].re, b.im - M2[ib].im);
    }
  return QPMS_SUCCESS;
}

// translations.h:158-166: the full sum.
int qpms_trans_calculator_get_AB_arrays_e32(const qpms_trans_calculator *c, qpms_complex_t *Adest, double *Aerr,
                                            qpms_complex_t *Bdest, double *Berr, ptrdiff_t deststride,
                                            ptrdiff_t srcstride, double eta, qpms_complex_t wavenumber, cart2_t b1,
                                            cart2_t b2, cart2_t beta, cart3_t particle_shift, double maxR,
                                            double maxK) {
  return qpms_trans_calculator_get_AB_arrays_e32_e(c, Adest, Aerr, Bdest, Berr, deststride, srcstride, eta,
                                                   wavenumber, b1, b2, beta, particle_shift, maxR, maxK, 7);
}

// Field of the periodic system at in-plane points (qpms_scatsyswk_scattered_E,
// scatsystem.c:2114-2188): batched over points, host buffers.
int qpms_gpu_scatsyswk_scattered_E(const qpms_scatsys_at_omega_k_t *sswk, qpms_bessel_t btyp,
                                   const qpms_complex_t *cvf, size_t npoints, const double *where_xyz,
                                   qpms_complex_t *E_xyz) {
  clear_error();
  if (!sswk || !sswk->ssw || !cvf || (npoints && (!where_xyz || !E_xyz))) { set_error("NULL argument"); return QPMS_EINVAL; }
  const qpms_scatsys_t *ss = sswk->ssw->ss;
  if (btyp != QPMS_HANKEL_PLUS) {
    set_error("Only scattered field with first kind Hankel functions currently implemented.");
    return QPMS_EINVAL;
  }
  if (ss->lattice_dimension != 2) { set_error("Only 2D-periodic lattices implemented"); return QPMS_EINVAL; }
  if (sswk->k[2] != 0) { set_error("Bloch vector must lie in the xy plane"); return QPMS_EINVAL; }
  const qg_c k = *(const qg_c *)&sswk->ssw->wavenumber;
  double eta = sswk->eta;
  if (eta == 0 || isnan(eta)) eta = qpms_ss_adjusted_eta(ss, sswk->ssw->wavenumber, sswk->k);
  const double beta[2] = {sswk->k[0], sswk->k[1]};
  return periodic_field(ss, k, beta, eta, (const qg_c *)cvf, npoints, where_xyz, (qg_c *)E_xyz);
}

// W, the lattice-summed translation matrix of the unit cell (scatsystem.c:1252-1281):
// the Ewald assembly with T = -1 gives I + W.
qpms_complex_t *qpms_scatsys_periodic_build_translation_matrix_full(qpms_complex_t *target, const qpms_scatsys_t *ss,
                                                                    qpms_complex_t wavenumber,
                                                                    const cart3_t *wavevector, double eta) {
  clear_error();
  if (!ss || !wavevector) { set_error("NULL argument"); return nullptr; }
  if (ss->lattice_dimension != 2) { set_error("Only 2D-periodic lattices implemented"); return nullptr; }
  if (wavevector->z != 0) { set_error("Only 2D xy-lattices currently supported"); return nullptr; }
  const double kv[3] = {wavevector->x, wavevector->y, 0.0};
  if (eta == 0 || isnan(eta)) eta = qpms_ss_adjusted_eta(ss, wavenumber, kv);
  const size_t N = ss->fecv_size;
  const int np = ss->p_count, n = (int)(N / np);
  std::vector<qg_c> T((size_t)ss->tm_count * n, cmk(-1.0, 0.0));
  const qg_c k = cmk(wavenumber.re, wavenumber.im);
  const double beta[2] = {kv[0], kv[1]};
  Dev dM;
  if (dalloc(dM, N * N * 16)) return nullptr;
  if (periodic_assemble_device(ss, 1, &k, T, 1, beta, &eta, dM.as<qg_c>(), 0)) return nullptr;
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

qpms_complex_t *qpms_scatsyswk_build_translation_matrix_full(qpms_complex_t *target,
                                                             const qpms_scatsys_at_omega_k_t *sswk) {
  clear_error();
  if (!sswk || !sswk->ssw) { set_error("NULL argument"); return nullptr; }
  cart3_t kv;
  kv.x = sswk->k[0];
  kv.y = sswk->k[1];
  kv.z = sswk->k[2];
  return qpms_scatsys_periodic_build_translation_matrix_full(target, sswk->ssw->ss, sswk->ssw->wavenumber, &kv,
                                                             sswk->eta);
}

ccart3_t qpms_scatsyswk_scattered_E(const qpms_scatsys_at_omega_k_t *sswk, qpms_bessel_t btyp,
                                    const qpms_complex_t *cvf, cart3_t where) {
  ccart3_t res;
  const double w[3] = {where.x, where.y, where.z};
  if (qpms_gpu_scatsyswk_scattered_E(sswk, btyp, cvf, 1, w, &res.x)) {
    qpms_complex_t nanc;
    nanc.re = nanc.im = NAN;
    res.x = res.y = res.z = nanc;
  }
  return res;
}

}  // extern "C"
