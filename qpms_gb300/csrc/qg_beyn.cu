// Beyn's contour-integral method for the nonlinear eigenproblem M(z) v = 0
// (the reference's beyn.c:69-86, 302-584, 625-667 and its scattering-system
// callers scatsystem.c:2280-2372).
//
// Per contour node z_i the matrix M(z_i) is built straight into device memory
// (assembly kernels for scattering systems, or one host->device copy for a
// user callback), factorised once by the dense solver (random butterfly +
// blocked LU, complex64 with FP64 iterative refinement, or plain complex128)
// and applied to the L probe columns; the quadrature sums
// A0 = sum dz X, A1 = sum dz (z - z0) X and their every-second-node coarse
// versions accumulate on the device.  The m x L results come back once; the
// SVD rank test, the L x L projected eigenproblem and the eigenvectors run on
// the host (qg_hostla.cu), exactly the steps of beyn_process_matrices.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <complex>
#include <vector>

#include "qg_assembly.h"
#include "qg_dense.h"
#include "qg_hostla.h"
#include "qg_internal.h"

namespace qg {
bool scatsys_is_own(const qpms_scatsys_t *ss);
bool scatsys_dense(const qpms_scatsys_t *ss);
int sym_pack_matrix_device(const qpms_scatsys_t *ss, int iri, const qg_c *dM, size_t ldm, qg_c *dout,
                           cudaStream_t st);
size_t sym_size(const qpms_scatsys_t *ss, int iri);
int sym_nirreps(const qpms_scatsys_t *ss);
void scatsys_tdiag(const qpms_scatsys_t *ss, int t, double om_re, double om_im, std::vector<qg_c> &out);
qg_c scatsys_wavenumber(const qpms_scatsys_t *ss, double om_re, double om_im);
int blas_handle_get(cublasHandle_t *h);
int assemble_modeproblem_device(const qpms_scatsys_t *ss, int nw, const std::vector<qg_c> &T_host, bool dense,
                                const std::vector<qg_c> &k_host, int J, qg_c *dM, cudaStream_t st);
int periodic_assemble_device(const qpms_scatsys_t *ss, int nw, const qg_c *k_host, const std::vector<qg_c> &T_host,
                             int nk, const double *beta_host, const double *eta_host, qg_c *dM, cudaStream_t st);

namespace {

typedef std::complex<double> cd;
inline cd to_cd(qpms_complex_t z) { return cd(z.re, z.im); }
inline qpms_complex_t from_cd(cd z) {
  qpms_complex_t r;
  r.re = z.real();
  r.im = z.imag();
  return r;
}

constexpr unsigned long long kDefaultSeed = 0x5eedbe11ULL;
constexpr double kDefaultRefineTol = 1e-12;
constexpr int kMaxRefine = 12;

struct BeynResultPriv {
  beyn_result_t pub;  // first member: callers see only this
  double max_node_resid = 0;
  int max_node_iters = 0;
  double quad_s = 0, total_s = 0;
};

struct DevPtr {
  void *p = nullptr;
  ~DevPtr() {
    if (p) cudaFree(p);
  }
};

// A0 += dz X, A1 += (z - z0) dz X, and twice each on even nodes for the coarse
// sums, in the order of beyn.c:567-580.
__global__ void beyn_accumulate_kernel(size_t n, const double2 *X, double2 dz, double2 dzz, int even, double2 *A0,
                                       double2 *A1, double2 *A0c, double2 *A1c) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const double2 x = X[t];
    const double2 a = make_double2(x.x * dz.x - x.y * dz.y, x.x * dz.y + x.y * dz.x);
    A0[t] = make_double2(A0[t].x + a.x, A0[t].y + a.y);
    if (even) {
      double2 c = A0c[t];
      c = make_double2(c.x + a.x, c.y + a.y);
      A0c[t] = make_double2(c.x + a.x, c.y + a.y);
    }
    const double2 b = make_double2(a.x * dzz.x - a.y * dzz.y, a.x * dzz.y + a.y * dzz.x);
    A1[t] = make_double2(A1[t].x + b.x, A1[t].y + b.y);
    if (even) {
      double2 c = A1c[t];
      c = make_double2(c.x + b.x, c.y + b.y);
      A1c[t] = make_double2(c.x + b.x, c.y + b.y);
    }
  }
}

// ---------------- sources of M(z), built column-major on the device ----------------
struct MSource {
  size_t m = 0;
  qg_c *stage = nullptr;  // row-major device staging buffer
  virtual ~MSource() {
    if (stage) cudaFree(stage);
  }
  int init_stage() {
    QG_CUDA_TRY(cudaMalloc(&stage, m * m * 16));
    return QPMS_SUCCESS;
  }
  // fills stage (row-major, the reference's layout)
  virtual int build_rowmajor(cd z, cudaStream_t st) = 0;
  int build(cd z, qg_c *dM, cudaStream_t st) {
    int e;
    if ((e = build_rowmajor(z, st))) return e;
    return launch_transpose(m, 1, stage, dM, st);
  }
};

struct CallbackSource : MSource {
  beyn_function_M_t f = nullptr;
  void *params = nullptr;
  qpms_complex_t *host = nullptr;  // pinned
  ~CallbackSource() override {
    if (host) cudaFreeHost(host);
  }
  int init() {
    int e;
    if ((e = init_stage())) return e;
    QG_CUDA_TRY(cudaHostAlloc((void **)&host, m * m * 16, cudaHostAllocDefault));
    return QPMS_SUCCESS;
  }
  int build_rowmajor(cd z, cudaStream_t st) override {
    QG_CUDA_TRY(cudaStreamSynchronize(st));  // the previous copy out of `host` has finished
    const int rc = f(host, m, from_cd(z), params);
    if (rc) {
      set_error("M(z) callback returned %d", rc);
      return rc;
    }
    QG_CUDA_TRY(cudaMemcpyAsync(stage, host, m * m * 16, cudaMemcpyHostToDevice, st));
    return QPMS_SUCCESS;
  }
};

// M(omega) = I - T S of a finite system (scatsystem.c:2280-2299), full or
// projected on irrep iri (assembled full, packed on the device).
struct FiniteSource : MSource {
  const qpms_scatsys_t *ss = nullptr;
  int iri = -1;
  qg_c *full = nullptr;  // N x N when packing
  ~FiniteSource() override {
    if (full) cudaFree(full);
  }
  int build_rowmajor(cd z, cudaStream_t st) override {
    std::vector<qg_c> T, d;
    for (int t = 0; t < ss->tm_count; ++t) {
      scatsys_tdiag(ss, t, z.real(), z.imag(), d);
      T.insert(T.end(), d.begin(), d.end());
    }
    std::vector<qg_c> k(1, scatsys_wavenumber(ss, z.real(), z.imag()));
    if (iri < 0) return assemble_modeproblem_device(ss, 1, T, scatsys_dense(ss), k, QPMS_HANKEL_PLUS, stage, st);
    const size_t N = ss->fecv_size;
    if (!full) QG_CUDA_TRY(cudaMalloc(&full, N * N * 16));
    int e;
    if ((e = assemble_modeproblem_device(ss, 1, T, scatsys_dense(ss), k, QPMS_HANKEL_PLUS, full, st))) return e;
    return sym_pack_matrix_device(ss, iri, full, N, stage, st);
  }
};

// M(omega) = I - T W(omega, k) of a 2D-periodic system (scatsystem.c:2332-2349)
struct PeriodicSource : MSource {
  const qpms_scatsys_t *ss = nullptr;
  double kvec[3] = {0, 0, 0};
  int build_rowmajor(cd z, cudaStream_t st) override {
    std::vector<qg_c> T, d;
    for (int t = 0; t < ss->tm_count; ++t) {
      scatsys_tdiag(ss, t, z.real(), z.imag(), d);
      T.insert(T.end(), d.begin(), d.end());
    }
    const qg_c k = scatsys_wavenumber(ss, z.real(), z.imag());
    qpms_complex_t kk;
    kk.re = k.re;
    kk.im = k.im;
    const double eta = qpms_ss_adjusted_eta(ss, kk, kvec);
    const double beta[2] = {kvec[0], kvec[1]};
    return periodic_assemble_device(ss, 1, &k, T, 1, beta, &eta, stage, st);
  }
};

// |M(z) v|_2 on the device
struct Residual {
  MSource *src = nullptr;
  size_t m = 0;
  qg_c *dM = nullptr;
  DevPtr dv, dy;
  int operator()(cd z, const cd *v, double *out) {
    cublasHandle_t h;
    int e;
    if ((e = blas_handle_get(&h))) return e;
    QG_BLAS_TRY(cublasSetStream(h, 0));
    if (!dv.p) QG_CUDA_TRY(cudaMalloc(&dv.p, m * 16));
    if (!dy.p) QG_CUDA_TRY(cudaMalloc(&dy.p, m * 16));
    if ((e = src->build(z, dM, 0))) return e;
    QG_CUDA_TRY(cudaMemcpy(dv.p, v, m * 16, cudaMemcpyHostToDevice));
    const cuDoubleComplex one = make_cuDoubleComplex(1, 0), zero = make_cuDoubleComplex(0, 0);
    QG_BLAS_TRY(cublasZgemv(h, CUBLAS_OP_N, (int)m, (int)m, &one, (const cuDoubleComplex *)dM, (int)m,
                            (const cuDoubleComplex *)dv.p, 1, &zero, (cuDoubleComplex *)dy.p, 1));
    double nrm = 0;
    QG_BLAS_TRY(cublasDznrm2(h, (int)m, (const cuDoubleComplex *)dy.p, 1, &nrm));
    g_launches.fetch_add(3);
    *out = nrm;
    return QPMS_SUCCESS;
  }
};

struct Processed {
  int K = 0;                 // retained eigenvalues
  std::vector<cd> eigval;    // K
  std::vector<cd> eigvec;    // K rows of length m
  std::vector<double> resid; // K
  std::vector<double> sigma; // l
};

// beyn_process_matrices (beyn.c:302-468): SVD rank test, B = V0^H A1 W0 Sigma^-1,
// eig(B), eigenvalues z0 + lambda, vectors V0 S, residual filter.
int process(const std::vector<cd> &A0, const std::vector<cd> &A1, size_t m, size_t l, cd z0, double rank_tol,
            size_t rank_sel_min, double res_tol, bool want_vec, Residual *resid, Processed &out) {
  std::vector<cd> U(m * l), V(l * l);
  out.sigma.assign(l, 0.0);
  if (hostla::svd_thin((int)m, (int)l, A0.data(), (int)m, U.data(), out.sigma.data(), V.data())) {
    set_error("Beyn: SVD did not converge");
    return QPMS_ERROR;
  }
  size_t K = 0;
  for (size_t k = 0; k < l; ++k)
    if (k < rank_sel_min || out.sigma[k] > rank_tol) ++K;
  out.K = 0;
  if (K == 0) return QPMS_SUCCESS;
  // TM2 = V0^H A1 (K x l), B = TM2 W0T^H (K x K), columns scaled by 1/sigma
  std::vector<cd> TM2(K * l), B(K * K), lam(K), S(K * K);
#pragma omp parallel for collapse(2) schedule(static)
  for (long b = 0; b < (long)l; ++b)
    for (long a = 0; a < (long)K; ++a) {
      cd acc = 0;
      const cd *u = &U[(size_t)a * m], *x = &A1[(size_t)b * m];
      for (size_t i = 0; i < m; ++i) acc += std::conj(u[i]) * x[i];
      TM2[a + b * K] = acc;
    }
  for (size_t c = 0; c < K; ++c)
    for (size_t a = 0; a < K; ++a) {
      cd acc = 0;
      for (size_t b = 0; b < l; ++b) acc += TM2[a + b * K] * V[b + c * l];
      B[a + c * K] = acc * (1.0 / out.sigma[c]);
    }
  if (hostla::eig((int)K, B.data(), (int)K, lam.data(), S.data())) {
    set_error("Beyn: eigenvalue iteration did not converge");
    return QPMS_ERROR;
  }
  std::vector<cd> V0S(m * K);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < (long)K; ++k)
    for (size_t i = 0; i < m; ++i) {
      cd acc = 0;
      for (size_t a = 0; a < K; ++a) acc += U[i + a * m] * S[a + k * K];
      V0S[i + k * m] = acc;
    }
  for (size_t k = 0; k < K; ++k) {
    const cd z = z0 + lam[k];
    double r = 0;
    if (res_tol > 0) {
      int e;
      if ((e = (*resid)(z, &V0S[k * m], &r))) return e;
      if (r > res_tol) continue;
    }
    out.eigval.push_back(z);
    out.resid.push_back(r);
    if (want_vec) out.eigvec.insert(out.eigvec.end(), V0S.begin() + k * m, V0S.begin() + (k + 1) * m);
    ++out.K;
  }
  return QPMS_SUCCESS;
}

unsigned grid1(size_t n) {
  size_t g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  return (unsigned)(g ? g : 1);
}

// Contour quadrature over nodes [nb, ne) (beyn.c:524-581): A0 = sum dz X,
// A1 = sum (z - z0) dz X, coarse sums over even node indices (global index),
// X = M(z)^-1 Vhat on the GPU.  Vh: host row-major m x l; outputs host
// column-major m x l.  Splitting the node range lets several processes or
// devices each sum a part; the parts add up to the full sums.
int beyn_quadrature(MSource &src, beyn_function_M_inv_Vhat_t minv, void *minv_params, size_t m, size_t l,
                    const beyn_contour_t *contour, size_t nb, size_t ne, const std::vector<cd> &Vh, int mode,
                    double refine_tol, unsigned long long seed, std::vector<cd> &A0, std::vector<cd> &A1,
                    std::vector<cd> &A0c, std::vector<cd> &A1c, double *max_res_out, int *max_it_out) {
  const size_t nml = m * l;
  std::vector<cd> Vc(nml);
  for (size_t i = 0; i < m; ++i)
    for (size_t j = 0; j < l; ++j) Vc[i + j * m] = Vh[i * l + j];
  DevPtr dV, dX, dA[4];
  if (cudaMalloc(&dV.p, nml * 16) != cudaSuccess || cudaMalloc(&dX.p, nml * 16) != cudaSuccess) {
    set_error("Beyn: out of device memory (m = %zu, l = %zu)", m, l);
    return QPMS_ENOMEM;
  }
  for (auto &a : dA)
    if (cudaMalloc(&a.p, nml * 16) != cudaSuccess || cudaMemset(a.p, 0, nml * 16) != cudaSuccess) {
      set_error("Beyn: out of device memory (m = %zu, l = %zu)", m, l);
      return QPMS_ENOMEM;
    }
  if (cudaMemcpy(dV.p, Vc.data(), nml * 16, cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error("Beyn: host to device copy failed");
    return QPMS_ERROR;
  }
  // the nodes run on a stream of their own (ordered with the legacy default
  // stream), so that the solver's repeated launch sequences can be captured
  // as CUDA graphs and replayed node after node
  struct Stream {
    cudaStream_t s = nullptr;
    ~Stream() {
      if (s) cudaStreamDestroy(s);
    }
  } ns;
  if (cudaStreamCreate(&ns.s) != cudaSuccess) {
    set_error("Beyn: stream creation failed");
    return QPMS_ERROR;
  }
  const cudaStream_t st = ns.s;
  DenseSolver ds;
  int e;
  if (!minv && (e = ds.init((int)m, (int)l, mode, seed ^ 0x9e3779b97f4a7c15ULL))) return e;
  ds.graphs = true;
  std::vector<qpms_complex_t> hx;
  double max_res = 0;
  int max_it = 0;
  const cd z0 = to_cd(contour->centre);
  for (size_t i = nb; i < ne; ++i) {
    const cd z = to_cd(contour->z_dz[i][0]), dz = to_cd(contour->z_dz[i][1]);
    if (minv) {  // user-supplied M(z)^-1 Vhat (row-major m x l)
      hx.resize(nml);
      const int rc = minv(hx.data(), m, l, (const qpms_complex_t *)Vh.data(), from_cd(z), minv_params);
      if (rc) {
        set_error("M^-1 Vhat callback returned %d", rc);
        return rc;
      }
      for (size_t r = 0; r < m; ++r)
        for (size_t c = 0; c < l; ++c) Vc[r + c * m] = to_cd(hx[r * l + c]);
      if (cudaMemcpy(dX.p, Vc.data(), nml * 16, cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("Beyn: host to device copy failed");
        return QPMS_ERROR;
      }
    } else {
      double res = 0;
      int it = 0;
      if ((e = src.build_rowmajor(z, st))) return e;
      // the staged row-major M(z) goes straight to the solver (transposed on the fly)
      if ((e = ds.factorize(src.stage, m, st, true))) return e;
      if ((e = ds.solve(src.stage, m, dV.p, dX.p, (int)l, refine_tol, kMaxRefine, &res, &it, st))) return e;
      if (!(res <= max_res)) max_res = res;  // NaN-propagating max
      if (it > max_it) max_it = it;
    }
    beyn_accumulate_kernel<<<grid1(nml), 256, 0, st>>>(nml, (const double2 *)dX.p, make_double2(dz.real(), dz.imag()),
                                                make_double2((z - z0).real(), (z - z0).imag()), (i % 2) == 0,
                                                (double2 *)dA[0].p, (double2 *)dA[1].p, (double2 *)dA[2].p,
                                                (double2 *)dA[3].p);
    if (cudaGetLastError() != cudaSuccess) {
      set_error("Beyn: accumulation kernel launch failed");
      return QPMS_ERROR;
    }
    g_launches.fetch_add(1);
  }
  A0.resize(nml);
  A1.resize(nml);
  A0c.resize(nml);
  A1c.resize(nml);
  if (cudaMemcpy(A0.data(), dA[0].p, nml * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(A1.data(), dA[1].p, nml * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(A0c.data(), dA[2].p, nml * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(A1c.data(), dA[3].p, nml * 16, cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("Beyn: device to host copy failed: %s", cudaGetErrorString(cudaGetLastError()));
    return QPMS_ERROR;
  }
  if (max_res_out) *max_res_out = max_res;
  if (max_it_out) *max_it_out = max_it;
  return QPMS_SUCCESS;
}

// Beyn steps 3-6 on the summed quadratures, coarse then fine, into a result
// (beyn.c:584-606).  resid may be NULL when res_tol <= 0.
BeynResultPriv *beyn_postprocess(Residual *resid, size_t m, size_t l, cd z0, const std::vector<cd> &A0,
                                 const std::vector<cd> &A1, const std::vector<cd> &A0c, const std::vector<cd> &A1c,
                                 double rank_tol, size_t rank_sel_min, double res_tol) {
  if (res_tol > 0 && !resid) {
    set_error("Beyn: residual filtering needs M(z)");
    return nullptr;
  }
  Processed coarse, fine;
  if (process(A0c, A1c, m, l, z0, rank_tol, rank_sel_min, res_tol, false, resid, coarse)) return nullptr;
  if (process(A0, A1, m, l, z0, rank_tol, rank_sel_min, res_tol, true, resid, fine)) return nullptr;
  BeynResultPriv *r = new (std::nothrow) BeynResultPriv();
  if (!r) {
    set_error("out of host memory");
    return nullptr;
  }
  beyn_result_t &p = r->pub;
  p.neig = fine.K;
  p.vlen = m;
  p.eigval = (qpms_complex_t *)calloc(l, 16);
  p.eigval_err = (qpms_complex_t *)calloc(l, 16);
  p.residuals = (double *)calloc(l, 8);
  p.eigvec = (qpms_complex_t *)calloc(l * m, 16);
  p.ranktest_SV = (double *)calloc(l > m ? l : m, 8);
  p.gsl = nullptr;
  if (!p.eigval || !p.eigval_err || !p.residuals || !p.eigvec || !p.ranktest_SV) {
    beyn_result_free(&p);
    set_error("out of host memory");
    return nullptr;
  }
  for (int k = 0; k < fine.K; ++k) {
    p.eigval[k] = from_cd(fine.eigval[k]);
    // error estimate: the coarse-contour eigenvalue nearest to this one
    cd best = 0;
    double bd = INFINITY;
    for (int j = 0; j < coarse.K; ++j) {
      const double d = std::abs(coarse.eigval[j] - fine.eigval[k]);
      if (d < bd) {
        bd = d;
        best = coarse.eigval[j];
      }
    }
    p.eigval_err[k] = from_cd(best - fine.eigval[k]);
    p.residuals[k] = fine.resid[k];
    for (size_t i = 0; i < m; ++i) p.eigvec[(size_t)k * m + i] = from_cd(fine.eigvec[(size_t)k * m + i]);
  }
  for (size_t k = 0; k < l; ++k) p.ranktest_SV[k] = fine.sigma[k];
  return r;
}

// Scale of the quadrature sums for a relative rank tolerance: sum |dz_i| times
// the RMS column norm of Vhat, the size A0 would have without cancellation
// when M^-1 is of order one on the contour.  With no eigenvalue inside, A0 is
// cancellation noise of about 1e-16 of it (the reference's absolute rank_tol
// cannot tell this from a mode when the frequencies are of order 1e15).
double rank_scale(const beyn_contour_t *contour, const std::vector<cd> &Vh, size_t l) {
  double s = 0, f = 0;
  for (size_t i = 0; i < contour->n; ++i) s += std::abs(to_cd(contour->z_dz[i][1]));
  for (const cd &v : Vh) f += std::norm(v);
  return s * sqrt(f / (double)l);
}

std::vector<cd> probe_or_given(size_t m, size_t l, const qpms_complex_t *Vhat, unsigned long long seed) {
  std::vector<cd> Vh(m * l);
  if (Vhat)
    for (size_t i = 0; i < m * l; ++i) Vh[i] = to_cd(Vhat[i]);
  else
    hostla::probe_matrix(m, l, seed, Vh.data());
  return Vh;
}

BeynResultPriv *beyn_core(MSource &src, beyn_function_M_inv_Vhat_t minv, void *minv_params, size_t m, size_t l,
                          const beyn_contour_t *contour, double rank_tol, size_t rank_sel_min, double res_tol,
                          const qpms_complex_t *Vhat, unsigned long long seed, int mode, double refine_tol) {
  const auto t0 = std::chrono::steady_clock::now();
  if (!contour || contour->n < 1 || m < 1 || l < 1 || l > m || (mode != 0 && mode != 1)) {
    set_error("Beyn: invalid arguments (need a contour, 1 <= l <= m, mode 0 or 1)");
    return nullptr;
  }
  if (refine_tol <= 0) refine_tol = kDefaultRefineTol;
  const std::vector<cd> Vh = probe_or_given(m, l, Vhat, seed);
  if (rank_tol < 0) rank_tol = -rank_tol * rank_scale(contour, Vh, l);
  std::vector<cd> A0, A1, A0c, A1c;
  double max_res = 0;
  int max_it = 0;
  if (beyn_quadrature(src, minv, minv_params, m, l, contour, 0, contour->n, Vh, mode, refine_tol, seed, A0, A1, A0c,
                      A1c, &max_res, &max_it))
    return nullptr;
  const auto t1 = std::chrono::steady_clock::now();
  DevPtr dM;
  Residual resid;
  if (res_tol > 0) {
    if (cudaMalloc(&dM.p, m * m * 16) != cudaSuccess) {
      set_error("Beyn: out of device memory for the residuals");
      return nullptr;
    }
    resid.src = &src;
    resid.m = m;
    resid.dM = (qg_c *)dM.p;
  }
  BeynResultPriv *r = beyn_postprocess(res_tol > 0 ? &resid : nullptr, m, l, to_cd(contour->centre), A0, A1, A0c,
                                       A1c, rank_tol, rank_sel_min, res_tol);
  if (!r) return nullptr;
  r->max_node_resid = max_res;
  r->max_node_iters = max_it;
  const auto t2 = std::chrono::steady_clock::now();
  r->quad_s = std::chrono::duration<double>(t1 - t0).count();
  r->total_s = std::chrono::duration<double>(t2 - t0).count();
  return r;
}

BeynResultPriv *scatsys_beyn(const qpms_scatsys_t *ss, const double *k, qpms_complex_t omega_centre,
                             double omega_rr, double omega_ri, size_t npoints, double rank_tol, size_t rank_sel_min,
                             double res_tol, size_t l, const qpms_complex_t *Vhat, unsigned long long seed, int mode,
                             double refine_tol, int iri = -1) {
  if (!ss || !scatsys_is_own(ss)) {
    set_error("Beyn on a scattering system needs one made by qpms_gpu_scatsys_create_spheres[_2d]");
    return nullptr;
  }
  if (k && ss->lattice_dimension != 2) {
    set_error("a Bloch vector needs a 2D-periodic system");
    return nullptr;
  }
  if (!k && ss->lattice_dimension != 0) {
    set_error("finite eigenmode search on a periodic system (give a Bloch vector)");
    return nullptr;
  }
  if (iri >= 0 && (k || iri >= sym_nirreps(ss))) {
    set_error(k ? "Irreps decomposition not yet supported for periodic systems"
                : "invalid irrep index (qpms_gpu_scatsys_set_symmetry gives the irreps)");
    return nullptr;
  }
  const size_t m = iri >= 0 ? sym_size(ss, iri) : ss->fecv_size;
  if (m == 0) {
    set_error("empty irrep");
    return nullptr;
  }
  beyn_contour_t *c = beyn_contour_ellipse(omega_centre, omega_rr, omega_ri, npoints);
  if (!c) return nullptr;
  FiniteSource fs;
  PeriodicSource ps;
  MSource *src = k ? (MSource *)&ps : (MSource *)&fs;
  fs.ss = ps.ss = ss;
  fs.iri = iri;
  if (k) {
    ps.kvec[0] = k[0];
    ps.kvec[1] = k[1];
    ps.kvec[2] = k[2];
  }
  src->m = m;
  BeynResultPriv *r = nullptr;
  if (!src->init_stage())
    r = beyn_core(*src, nullptr, nullptr, m, l ? l : m, c, rank_tol, rank_sel_min, res_tol, Vhat, seed, mode,
                  refine_tol);
  free(c);
  return r;
}

bool ellipse_inside(beyn_contour_t *c, qpms_complex_t z) {
  // beyn.c:61-67: the half-axes sit in the entry after the last node
  const double rRe = c->z_dz[c->n][0].re, rIm = c->z_dz[c->n][1].re;
  const double x = (z.re - c->centre.re) / rRe, y = (z.im - c->centre.im) / rIm;
  return x * x + y * y < 1;
}

}  // namespace
}  // namespace qg

using namespace qg;

extern "C" {

beyn_contour_t *beyn_contour_ellipse(qpms_complex_t centre, double rRe, double rIm, size_t n) {
  beyn_contour_t *c = (beyn_contour_t *)malloc(sizeof(beyn_contour_t) + (n + 1) * sizeof(c->z_dz[0]));
  if (!c) {
    set_error("out of host memory");
    return nullptr;
  }
  c->centre = centre;
  c->n = n;
  for (size_t i = 0; i < n; ++i) {
    const double t = i * 2 * M_PI / n;
    const double st = sin(t), ct = cos(t);
    c->z_dz[i][0].re = centre.re + ct * rRe;
    c->z_dz[i][0].im = centre.im + st * rIm;
    c->z_dz[i][1].re = -rRe * st * (2 * M_PI / n);
    c->z_dz[i][1].im = rIm * ct * (2 * M_PI / n);
  }
  c->z_dz[n][0].re = rRe;
  c->z_dz[n][0].im = 0;
  c->z_dz[n][1].re = rIm;
  c->z_dz[n][1].im = 0;
  c->inside_test = ellipse_inside;
  return c;
}

void beyn_result_free(beyn_result_t *r) {
  if (!r) return;
  free(r->eigval);
  free(r->eigval_err);
  free(r->residuals);
  free(r->eigvec);
  free(r->ranktest_SV);
  delete reinterpret_cast<BeynResultPriv *>(r);
}

beyn_result_t *qpms_gpu_beyn_solve(size_t m, size_t l, beyn_function_M_t M, void *params,
                                   const beyn_contour_t *contour, double rank_tol, size_t rank_sel_min,
                                   double res_tol, const qpms_complex_t *Vhat, unsigned long long seed, int mode,
                                   double refine_tol) {
  clear_error();
  if (!M) {
    set_error("Beyn: NULL M function");
    return nullptr;
  }
  CallbackSource src;
  src.m = m;
  src.f = M;
  src.params = params;
  if (m < 1 || src.init()) {
    if (m < 1) set_error("Beyn: m must be positive");
    return nullptr;
  }
  BeynResultPriv *r =
      beyn_core(src, nullptr, nullptr, m, l, contour, rank_tol, rank_sel_min, res_tol, Vhat, seed, mode, refine_tol);
  return r ? &r->pub : nullptr;
}

beyn_result_t *beyn_solve(size_t m, size_t l, beyn_function_M_t M, beyn_function_M_inv_Vhat_t M_inv_Vhat,
                          void *params, const beyn_contour_t *contour, double rank_tol, size_t rank_sel_min,
                          double res_tol) {
  clear_error();
  // the reference's rank test is absolute; negative values (the extended
  // entry points' relative test) keep every singular value there
  if (rank_tol < 0) rank_tol = 0;
  if (!M_inv_Vhat)
    return qpms_gpu_beyn_solve(m, l, M, params, contour, rank_tol, rank_sel_min, res_tol, nullptr, kDefaultSeed, 1,
                               kDefaultRefineTol);
  if (!M) {
    set_error("Beyn: NULL M function");
    return nullptr;
  }
  CallbackSource src;  // used for the residuals only
  src.m = m;
  src.f = M;
  src.params = params;
  if (m < 1 || src.init()) {
    if (m < 1) set_error("Beyn: m must be positive");
    return nullptr;
  }
  BeynResultPriv *r = beyn_core(src, M_inv_Vhat, params, m, l, contour, rank_tol, rank_sel_min, res_tol, nullptr,
                                kDefaultSeed, 1, kDefaultRefineTol);
  return r ? &r->pub : nullptr;
}

beyn_result_t *qpms_gpu_scatsys_find_eigenmodes(const qpms_scatsys_t *ss, const double *k,
                                                qpms_complex_t omega_centre, double omega_rr, double omega_ri,
                                                size_t contour_npoints, double rank_tol, size_t rank_sel_min,
                                                double res_tol, size_t l, const qpms_complex_t *Vhat,
                                                unsigned long long seed, int mode, double refine_tol) {
  clear_error();
  BeynResultPriv *r = scatsys_beyn(ss, k, omega_centre, omega_rr, omega_ri, contour_npoints, rank_tol, rank_sel_min,
                                   res_tol, l, Vhat, seed, mode, refine_tol);
  return r ? &r->pub : nullptr;
}

beyn_result_t *qpms_scatsys_finite_find_eigenmodes(const qpms_scatsys_t *ss, qpms_iri_t iri,
                                                   qpms_complex_t omega_centre, double omega_rr, double omega_ri,
                                                   size_t contour_npoints, double rank_tol, size_t rank_sel_min,
                                                   double res_tol) {
  clear_error();
  // iri: QPMS_NO_IRREP for the full system, else M projected on the irrep
  // (eigenvectors in the packed basis); absolute rank test as the reference's
  if (rank_tol < 0) rank_tol = 0;
  BeynResultPriv *r = scatsys_beyn(ss, nullptr, omega_centre, omega_rr, omega_ri, contour_npoints, rank_tol,
                                   rank_sel_min, res_tol, 0, nullptr, kDefaultSeed, 1, kDefaultRefineTol,
                                   iri == QPMS_NO_IRREP ? -1 : iri);
  return r ? &r->pub : nullptr;
}

// The extended finite search on one irrep (probe columns, probe matrix or
// seed, precision mode, refinement tolerance as qpms_gpu_scatsys_find_eigenmodes).
beyn_result_t *qpms_gpu_scatsys_find_eigenmodes_irrep(const qpms_scatsys_t *ss, int iri, qpms_complex_t omega_centre,
                                                      double omega_rr, double omega_ri, size_t contour_npoints,
                                                      double rank_tol, size_t rank_sel_min, double res_tol, size_t l,
                                                      const qpms_complex_t *Vhat, unsigned long long seed, int mode,
                                                      double refine_tol) {
  clear_error();
  if (iri < 0) {
    set_error("invalid irrep index %d", iri);
    return nullptr;
  }
  BeynResultPriv *r = scatsys_beyn(ss, nullptr, omega_centre, omega_rr, omega_ri, contour_npoints, rank_tol,
                                   rank_sel_min, res_tol, l, Vhat, seed, mode, refine_tol, iri);
  return r ? &r->pub : nullptr;
}

beyn_result_t *qpms_scatsys_periodic_find_eigenmodes(const qpms_scatsys_t *ss, const double k[3],
                                                     qpms_complex_t omega_centre, double omega_rr, double omega_ri,
                                                     size_t contour_npoints, double rank_tol, size_t rank_sel_min,
                                                     double res_tol) {
  clear_error();
  if (!k) {
    set_error("NULL Bloch vector");
    return nullptr;
  }
  if (rank_tol < 0) rank_tol = 0;  // absolute rank test as the reference's
  BeynResultPriv *r = scatsys_beyn(ss, k, omega_centre, omega_rr, omega_ri, contour_npoints, rank_tol, rank_sel_min,
                                   res_tol, 0, nullptr, kDefaultSeed, 1, kDefaultRefineTol);
  return r ? &r->pub : nullptr;
}

int qpms_gpu_scatsys_beyn_quadrature(const qpms_scatsys_t *ss, const double *k, const beyn_contour_t *contour,
                                     size_t node_begin, size_t node_end, size_t l, const qpms_complex_t *Vhat,
                                     unsigned long long seed, int mode, double refine_tol, qpms_complex_t *A0,
                                     qpms_complex_t *A1, qpms_complex_t *A0c, qpms_complex_t *A1c) {
  clear_error();
  if (!ss || !scatsys_is_own(ss) || !contour || !A0 || !A1 || !A0c || !A1c || node_begin > node_end ||
      node_end > contour->n || (mode != 0 && mode != 1)) {
    set_error("invalid arguments");
    return QPMS_EINVAL;
  }
  if ((k && ss->lattice_dimension != 2) || (!k && ss->lattice_dimension != 0)) {
    set_error("a Bloch vector goes with a 2D-periodic system, none with a finite one");
    return QPMS_EINVAL;
  }
  const size_t m = ss->fecv_size;
  if (l < 1 || l > m) {
    set_error("1 <= l <= fecv_size");
    return QPMS_EINVAL;
  }
  FiniteSource fs;
  PeriodicSource ps;
  MSource *src = k ? (MSource *)&ps : (MSource *)&fs;
  fs.ss = ps.ss = ss;
  if (k) {
    ps.kvec[0] = k[0];
    ps.kvec[1] = k[1];
    ps.kvec[2] = k[2];
  }
  src->m = m;
  int e;
  if ((e = src->init_stage())) return e;
  const std::vector<cd> Vh = probe_or_given(m, l, Vhat, seed);
  std::vector<cd> a0, a1, a0c, a1c;
  if ((e = beyn_quadrature(*src, nullptr, nullptr, m, l, contour, node_begin, node_end, Vh, mode,
                           refine_tol > 0 ? refine_tol : kDefaultRefineTol, seed, a0, a1, a0c, a1c, nullptr,
                           nullptr)))
    return e;
  for (size_t i = 0; i < m * l; ++i) {
    A0[i] = from_cd(a0[i]);
    A1[i] = from_cd(a1[i]);
    A0c[i] = from_cd(a0c[i]);
    A1c[i] = from_cd(a1c[i]);
  }
  return QPMS_SUCCESS;
}

beyn_result_t *qpms_gpu_beyn_process(size_t m, size_t l, const qpms_complex_t *A0, const qpms_complex_t *A1,
                                     const qpms_complex_t *A0c, const qpms_complex_t *A1c, qpms_complex_t z0,
                                     double rank_tol, size_t rank_sel_min) {
  clear_error();
  if (!A0 || !A1 || !A0c || !A1c || m < 1 || l < 1 || l > m) {
    set_error("invalid arguments");
    return nullptr;
  }
  std::vector<cd> a0(m * l), a1(m * l), a0c(m * l), a1c(m * l);
  for (size_t i = 0; i < m * l; ++i) {
    a0[i] = to_cd(A0[i]);
    a1[i] = to_cd(A1[i]);
    a0c[i] = to_cd(A0c[i]);
    a1c[i] = to_cd(A1c[i]);
  }
  BeynResultPriv *r = beyn_postprocess(nullptr, m, l, to_cd(z0), a0, a1, a0c, a1c, rank_tol, rank_sel_min, 0.0);
  return r ? &r->pub : nullptr;
}

int qpms_gpu_beyn_result_stats(const beyn_result_t *result, double *max_node_resid, int *max_node_iters,
                               double *quadrature_s, double *total_s) {
  if (!result) return QPMS_EINVAL;
  const BeynResultPriv *r = reinterpret_cast<const BeynResultPriv *>(result);
  if (max_node_resid) *max_node_resid = r->max_node_resid;
  if (max_node_iters) *max_node_iters = r->max_node_iters;
  if (quadrature_s) *quadrature_s = r->quad_s;
  if (total_s) *total_s = r->total_s;
  return QPMS_SUCCESS;
}

int qpms_gpu_beyn_probe_matrix(size_t m, size_t l, unsigned long long seed, qpms_complex_t *out) {
  if (!out) return QPMS_EINVAL;
  std::vector<cd> v(m * l);
  hostla::probe_matrix(m, l, seed, v.data());
  for (size_t i = 0; i < m * l; ++i) out[i] = from_cd(v[i]);
  return QPMS_SUCCESS;
}

int qpms_gpu_host_svd(int m, int n, const qpms_complex_t *A, qpms_complex_t *U, double *s, qpms_complex_t *V) {
  if (m < n || n < 1 || !A || !U || !s || !V) return QPMS_EINVAL;
  return hostla::svd_thin(m, n, (const cd *)A, m, (cd *)U, s, (cd *)V) ? QPMS_ERROR : QPMS_SUCCESS;
}

int qpms_gpu_host_eig(int n, const qpms_complex_t *A, qpms_complex_t *w, qpms_complex_t *X) {
  if (n < 1 || !A || !w || !X) return QPMS_EINVAL;
  return hostla::eig(n, (const cd *)A, n, (cd *)w, (cd *)X) ? QPMS_ERROR : QPMS_SUCCESS;
}

}  // extern "C"
