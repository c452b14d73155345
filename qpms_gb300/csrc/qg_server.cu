// Mode-problem serving loop: continuous batching of scattering solves on one GPU.
//
// A request is one plane-wave scattering solve of a finite cluster or of a
// 2D-periodic lattice at one (omega[, Bloch vector]) -- the unit of work of
// the reference's scatter scripts (misc/finiterectlat-scatter.py,
// misc/infiniterectlat-scatter.py) over scatsystem.c:1180-1357 and 2202-2273.
// Requests arrive at any time; worker threads (one CUDA stream each) take
// work as HBM and workers free up:
//   * large systems (N > kSmallN) run alone: assembly kernel -> dense solver
//     (random butterfly + blocked LU on the tensor cores, complex64 with FP64
//     refinement, or complex128) -> sigma_ext;
//   * small systems (lattice unit cells, small clusters) of the same system
//     are gathered into one batch: paired (omega, k) Ewald or finite assembly
//     for the whole batch -> batched LU -> refinement -> sigma_ext.
// Admission is by device-memory footprint against a budget; a request that
// does not fit waits while smaller ones behind it may pass (a bounded number
// of times, so it cannot starve).  Device memory comes from a private
// stream-ordered pool, so steady-state allocation never synchronises the
// device and the workers' kernels overlap.  The per-lMax translation tables
// are resident (shared calculators); per-system particle data are uploaded
// once and kept, keyed by content.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "qg_assembly.h"
#include "qg_batched.h"
#include "qg_dense.h"
#include "qg_ewald.h"
#include "qg_internal.h"

namespace qg {
bool scatsys_is_own(const qpms_scatsys_t *ss);
int scatsys_lmax(const qpms_scatsys_t *ss);
bool scatsys_dense(const qpms_scatsys_t *ss);
void scatsys_tdiag(const qpms_scatsys_t *ss, int t, double om_re, double om_im, std::vector<qg_c> &out);
qg_c scatsys_wavenumber(const qpms_scatsys_t *ss, double om_re, double om_im);
void planewave_direction_coeffs(int lMax, const double k_dir[3], const qpms_complex_t E_cart[3],
                                std::vector<qg_c> &coef);
int blas_handle_get(cublasHandle_t *h);
int ewald_assemble_locked(const qpms_scatsys_t *ss, const EwaldArgs &a, cudaStream_t st);
int ewald_assemble_dense(const qpms_scatsys_t *ss, const EwaldArgs &a, int n, cudaStream_t st);
int layered_system(const qpms_scatsys_t *ss);
}  // namespace qg

using namespace qg;

struct qpms_gpu_server;

namespace {

constexpr size_t kSmallN = 256;     // systems up to this size go through the batched path
constexpr int kMaxBatch = 256;      // requests per batch
constexpr int kMaxSkips = 8;        // times a waiting request may be overtaken
constexpr double kRefineTol = 1e-11;  // results are promised at a 1e-10 relative residual: a tenfold margin
constexpr int kMaxRefine = 12;

struct Job {
  uint64_t id = 0;
  qpms_gpu_request_t req;
  qpms_complex_t *f_out = nullptr;
  size_t N = 0, bytes = 0;
  bool small = false, periodic = false;
  int skips = 0;
  qpms_gpu_result_t res;
  std::string err;
  bool done = false;
};

struct SysDev {
  double *pos = nullptr;
  int *tmid = nullptr;
};

// allocations still to fail on purpose (qpms_gpu_server_testing_fail_allocations)
std::atomic<int> g_fail_allocs{0};

bool injected_failure() {
  int n = g_fail_allocs.load();
  while (n > 0)
    if (g_fail_allocs.compare_exchange_weak(n, n - 1)) return true;
  return false;
}

// device buffers of one job or batch, returned to the pool on destruction
struct PoolBufs {
  cudaStream_t st;
  std::vector<void *> ptrs;
  explicit PoolBufs(cudaStream_t s) : st(s) {}
  ~PoolBufs() {
    for (void *p : ptrs) cudaFreeAsync(p, st);
  }
  template <typename T>
  int get(T **out, size_t bytes, cudaMemPool_t pool) {
    void *p = nullptr;
    if (injected_failure()) {
      set_error("server: device pool allocation of %zu bytes failed (injected)", bytes);
      return QPMS_ENOMEM;
    }
    if (cudaMallocFromPoolAsync(&p, bytes ? bytes : 16, pool, st) != cudaSuccess) {
      set_error("server: device pool allocation of %zu bytes failed", bytes);
      return QPMS_ENOMEM;
    }
    ptrs.push_back(p);
    *out = (T *)p;
    return QPMS_SUCCESS;
  }
};

double secs(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

uint64_t fnv(const void *data, size_t n, uint64_t h = 1469598103934665603ULL) {
  const unsigned char *p = (const unsigned char *)data;
  for (size_t i = 0; i < n; ++i) h = (h ^ p[i]) * 1099511628211ULL;
  return h;
}

}  // namespace

struct qpms_gpu_server {
  int device = 0, mode = 1, nworkers = 1;
  size_t budget = 0, in_use = 0, peak = 0;
  cudaMemPool_t pool = nullptr;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job *> pending;
  std::unordered_map<uint64_t, Job *> jobs;
  uint64_t next_id = 1;
  bool stop = false;
  int busy = 0, max_busy = 0;
  size_t completed = 0, batches = 0;
  std::vector<std::thread> workers;
  std::mutex sys_mu;
  std::unordered_map<uint64_t, SysDev> sys;  // keyed by a hash of the particle data
  std::vector<void *> sys_ptrs;

  double now() const { return secs(t0, std::chrono::steady_clock::now()); }

  size_t job_bytes(const Job &j) const {
    const size_t N = j.N;
    if (j.small) return N * N * 16 + batched_solve_bytes(1, N, mode) + 8 * N * 16 + 4096;
    return N * N * 16 + DenseSolver::footprint((int)N, 1, mode) + 8 * N * 16 + 4096;
  }

  // particle positions and T-matrix ids, uploaded once per distinct system
  int system_dev(const qpms_scatsys_t *ss, cudaStream_t st, SysDev *out) {
    const int np = ss->p_count;
    std::vector<double> pos(3 * np);
    std::vector<int> tm(np);
    for (int i = 0; i < np; ++i) {
      pos[3 * i] = ss->p[i].pos.x;
      pos[3 * i + 1] = ss->p[i].pos.y;
      pos[3 * i + 2] = ss->p[i].pos.z;
      tm[i] = ss->p[i].tmatrix_id;
    }
    uint64_t key = fnv(pos.data(), pos.size() * 8);
    key = fnv(tm.data(), tm.size() * 4, key);
    key = fnv(&np, sizeof np, key);
    std::lock_guard<std::mutex> lk(sys_mu);
    auto it = sys.find(key);
    if (it != sys.end()) {
      *out = it->second;
      return QPMS_SUCCESS;
    }
    SysDev d;
    if (cudaMallocFromPoolAsync((void **)&d.pos, pos.size() * 8, pool, st) != cudaSuccess ||
        cudaMallocFromPoolAsync((void **)&d.tmid, tm.size() * 4 + 4, pool, st) != cudaSuccess) {
      set_error("server: device pool allocation failed");
      return QPMS_ENOMEM;
    }
    sys_ptrs.push_back(d.pos);
    sys_ptrs.push_back(d.tmid);
    QG_CUDA_TRY(cudaMemcpyAsync(d.pos, pos.data(), pos.size() * 8, cudaMemcpyHostToDevice, st));
    QG_CUDA_TRY(cudaMemcpyAsync(d.tmid, tm.data(), tm.size() * 4, cudaMemcpyHostToDevice, st));
    QG_CUDA_TRY(cudaStreamSynchronize(st));  // visible to every worker's stream from here on
    sys[key] = d;
    *out = d;
    return QPMS_SUCCESS;
  }

  // ---- scheduling (called with mu held) ----
  bool fits(size_t b) const { return in_use + b <= budget; }

  // a batch of small jobs of the same system as `first`, in arrival order
  void gather(Job *first, std::vector<Job *> &out, size_t &bytes) {
    out.clear();
    bytes = 0;
    for (Job *j : pending) {
      if (!j->small || j->req.ss != first->req.ss) continue;
      if ((int)out.size() >= kMaxBatch || !fits(bytes + j->bytes)) break;
      out.push_back(j);
      bytes += j->bytes;
    }
  }

  bool pick(std::vector<Job *> &work, size_t &bytes) {
    if (pending.empty()) return false;
    Job *head = pending.front();
    auto take = [&](Job *j) -> bool {
      if (j->small) {
        gather(j, work, bytes);
        return !work.empty() && work.front() == j;
      }
      if (!fits(j->bytes)) return false;
      work.assign(1, j);
      bytes = j->bytes;
      return true;
    };
    if (take(head)) return true;
    if (head->skips >= kMaxSkips) return false;  // it waits for memory; nobody overtakes it any more
    for (Job *j : pending) {
      if (j == head) continue;
      if (take(j)) {
        ++head->skips;
        return true;
      }
    }
    return false;
  }

  void worker_main() {
    cudaSetDevice(device);
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return;
    std::vector<Job *> work;
    for (;;) {
      size_t bytes = 0;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || pick(work, bytes); });
        if (stop && work.empty()) break;
        if (work.empty()) continue;
        for (Job *j : work) {
          pending.erase(std::find(pending.begin(), pending.end(), j));
          j->res.t_start = now();
          j->res.batch_size = (int)work.size();
        }
        in_use += bytes;
        peak = std::max(peak, in_use);
        ++busy;
        max_busy = std::max(max_busy, busy);
        ++batches;
      }
      clear_error();
      const int rc = work.front()->small ? run_batch(work, st) : run_large(work.front(), st);
      const std::string msg = rc ? std::string(qpms_gpu_last_error()) : std::string();
      {
        std::lock_guard<std::mutex> lk(mu);
        const double t = now();
        for (Job *j : work) {
          j->res.t_done = t;
          if (rc) {
            j->res.status = rc;
            j->err = msg;
          }
          j->done = true;
        }
        in_use -= bytes;
        --busy;
        completed += work.size();
        work.clear();
      }
      cv_done.notify_all();
      cv_work.notify_all();
    }
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }

  // ---- one large finite or periodic system: dense solver ----
  int run_large(Job *j, cudaStream_t st) {
    const qpms_scatsys_t *ss = j->req.ss;
    const int lMax = scatsys_lmax(ss), np = ss->p_count, ntm = ss->tm_count, n = 2 * lMax * (lMax + 2);
    const size_t N = j->N;
    std::vector<qg_c> T, d, coef;
    for (int t = 0; t < ntm; ++t) {
      scatsys_tdiag(ss, t, j->req.omega, 0.0, d);
      T.insert(T.end(), d.begin(), d.end());
    }
    const qg_c k = scatsys_wavenumber(ss, j->req.omega, 0.0);
    double kvec[3];
    if (incidence(j, k, lMax, kvec, coef)) return QPMS_EINVAL;
    SysDev sd;
    int e;
    if ((e = system_dev(ss, st, &sd))) return e;
    cublasHandle_t h;
    if ((e = blas_handle_get(&h))) return e;
    QG_BLAS_TRY(cublasSetStream(h, st));
    PoolBufs B(st);
    qg_c *dM, *dT, *dk, *dcoef, *da, *db, *dx;
    double *dkv, *dsig, *dbeta, *deta;
    int *derr;
    if ((e = B.get(&dM, N * N * 16, pool)) || (e = B.get(&dT, T.size() * 16, pool)) || (e = B.get(&dk, 16, pool)) ||
        (e = B.get(&dcoef, coef.size() * 16, pool)) || (e = B.get(&da, N * 16, pool)) ||
        (e = B.get(&db, N * 16, pool)) || (e = B.get(&dx, N * 16, pool)) || (e = B.get(&dkv, 24, pool)) ||
        (e = B.get(&dsig, 8, pool)) || (e = B.get(&dbeta, 16, pool)) || (e = B.get(&deta, 8, pool)) ||
        (e = B.get(&derr, 4, pool)))
      return e;
    QG_CUDA_TRY(cudaMemcpyAsync(dT, T.data(), T.size() * 16, cudaMemcpyHostToDevice, st));
    QG_CUDA_TRY(cudaMemcpyAsync(dk, &k, 16, cudaMemcpyHostToDevice, st));
    QG_CUDA_TRY(cudaMemcpyAsync(dcoef, coef.data(), coef.size() * 16, cudaMemcpyHostToDevice, st));
    QG_CUDA_TRY(cudaMemcpyAsync(dkv, kvec, 24, cudaMemcpyHostToDevice, st));
    if ((e = assemble(j->periodic, ss, 1, sd, dT, dk, &j->req, &k, dbeta, deta, derr, dM, st))) return e;
    if ((e = launch_incident(1, np, n, dcoef, dkv, sd.pos, da, st))) return e;
    if ((e = launch_apply_t(1, np, n, ntm, scatsys_dense(ss) ? 1 : 0, sd.tmid, dT, da, db, st))) return e;
    DenseSolver ds;
    double res = 0;
    int it = 0;
    // with several workers the diagonal-block inversions already overlap other
    // requests' work; the LU's own lookahead then only costs launches
    // (measured on the serving trace: 94.5 solves/s with it, 100.7 without)
    // (also measured: lookahead only for requests above 4,096 / 8,192 / 12,000
    // unknowns, 106-109 solves/s against 116 without)
    ds.lookahead = nworkers == 1;
    // and 128-wide blocks at every size: the trailing updates, not the
    // inversion chain, bound a loaded server (107.5 solves/s against 104.4
    // with the single-solve tuning's 64-wide blocks below 6144 unknowns)
    ds.nb_pref = 128;
    // and the substitutions as one launch per block and sweep: the one-launch
    // sweeps' waiting warps hold SM slots the other requests' kernels could
    // use (135.4 / 135.6 solves/s with them, 138.2 / 137.7 without, 8 workers)
    ds.sweeps = nworkers == 1;
    // and groups of 3 blocks in the LU: without the lookahead the in-group
    // inversions cost nothing extra here (136.0 / 137.0 solves/s with pairs,
    // 138.1 with groups of 3, 138.2 / 137.0 with groups of 4)
    ds.group = nworkers == 1 ? 2 : 3;
    if ((e = ds.init((int)N, 1, mode, 0x5eed ^ j->id, pool, st))) return e;
    if ((e = ds.factorize(dM, N, st, true))) return e;
    if ((e = ds.solve(dM, N, db, dx, 1, kRefineTol, kMaxRefine, &res, &it, st))) return e;
    j->res.fallback = ds.refactors > 0 ? 1 : 0;
    if ((e = launch_sigma_ext(1, N, da, dx, dk, dsig, st))) return e;
    double sig = 0;
    QG_CUDA_TRY(cudaMemcpyAsync(&sig, dsig, 8, cudaMemcpyDeviceToHost, st));
    if (j->f_out) QG_CUDA_TRY(cudaMemcpyAsync(j->f_out, dx, N * 16, cudaMemcpyDeviceToHost, st));
    QG_CUDA_TRY(cudaStreamSynchronize(st));
    j->res.sigma_ext = sig;
    j->res.residual = res;
    j->res.iters = it;
    return QPMS_SUCCESS;
  }

  // ---- a batch of small systems (all the same scattering system) ----
  int run_batch(std::vector<Job *> &work, cudaStream_t st) {
    const qpms_scatsys_t *ss = work.front()->req.ss;
    const bool periodic = work.front()->periodic;
    const int lMax = scatsys_lmax(ss), np = ss->p_count, ntm = ss->tm_count, n = 2 * lMax * (lMax + 2);
    const size_t N = work.front()->N;
    const int nb = (int)work.size();
    std::vector<qg_c> T, d, coefs, ks(nb), cf;
    std::vector<double> kv(3 * nb), beta(2 * nb), eta(nb);
    for (int b = 0; b < nb; ++b) {
      Job *j = work[b];
      for (int t = 0; t < ntm; ++t) {
        scatsys_tdiag(ss, t, j->req.omega, 0.0, d);
        T.insert(T.end(), d.begin(), d.end());
      }
      ks[b] = scatsys_wavenumber(ss, j->req.omega, 0.0);
      if (incidence(j, ks[b], lMax, &kv[3 * b], cf)) return QPMS_EINVAL;
      coefs.insert(coefs.end(), cf.begin(), cf.end());
      if (periodic) {
        const double kk[3] = {j->req.k[0], j->req.k[1], 0.0};
        qpms_complex_t kc;
        kc.re = ks[b].re;
        kc.im = ks[b].im;
        eta[b] = qpms_ss_adjusted_eta(ss, kc, kk);
        beta[2 * b] = kk[0];
        beta[2 * b + 1] = kk[1];
      }
    }
    SysDev sd;
    int e;
    if ((e = system_dev(ss, st, &sd))) return e;
    cublasHandle_t h;
    if ((e = blas_handle_get(&h))) return e;
    PoolBufs B(st);
    qg_c *dM, *dT, *dk, *dcoef, *da, *db, *dx;
    double *dkv, *dsig, *dbeta, *deta;
    int *derr;
    void *scratch;
    if ((e = B.get(&dM, nb * N * N * 16, pool)) || (e = B.get(&dT, T.size() * 16, pool)) ||
        (e = B.get(&dk, nb * 16, pool)) || (e = B.get(&dcoef, coefs.size() * 16, pool)) ||
        (e = B.get(&da, nb * N * 16, pool)) || (e = B.get(&db, nb * N * 16, pool)) ||
        (e = B.get(&dx, nb * N * 16, pool)) || (e = B.get(&dkv, nb * 24, pool)) || (e = B.get(&dsig, nb * 8, pool)) ||
        (e = B.get(&dbeta, nb * 16, pool)) || (e = B.get(&deta, nb * 8, pool)) || (e = B.get(&derr, 4, pool)) ||
        (e = B.get(&scratch, batched_solve_bytes(nb, N, mode), pool)))
      return e;
    QG_CUDA_TRY(cudaMemcpyAsync(dT, T.data(), T.size() * 16, cudaMemcpyHostToDevice, st));
    QG_CUDA_TRY(cudaMemcpyAsync(dk, ks.data(), nb * 16, cudaMemcpyHostToDevice, st));
    QG_CUDA_TRY(cudaMemcpyAsync(dcoef, coefs.data(), coefs.size() * 16, cudaMemcpyHostToDevice, st));
    QG_CUDA_TRY(cudaMemcpyAsync(dkv, kv.data(), nb * 24, cudaMemcpyHostToDevice, st));
    QG_CUDA_TRY(cudaMemcpyAsync(dbeta, beta.data(), nb * 16, cudaMemcpyHostToDevice, st));
    QG_CUDA_TRY(cudaMemcpyAsync(deta, eta.data(), nb * 8, cudaMemcpyHostToDevice, st));
    if ((e = assemble(periodic, ss, nb, sd, dT, dk, nullptr, nullptr, dbeta, deta, derr, dM, st))) return e;
    if ((e = launch_incident(nb, np, n, dcoef, dkv, sd.pos, da, st, (size_t)n))) return e;
    if ((e = launch_apply_t(nb, np, n, ntm, scatsys_dense(ss) ? 1 : 0, sd.tmid, dT, da, db, st))) return e;
    std::vector<double> res(nb), sig(nb);
    std::vector<int> its(nb), info(nb), fb(nb);
    if ((e = batched_solve(h, st, nb, N, dM, db, dx, mode, kRefineTol, kMaxRefine, scratch, res.data(), its.data(),
                           info.data(), nullptr, fb.data())))
      return e;
    if ((e = launch_sigma_ext(nb, N, da, dx, dk, dsig, st))) return e;
    QG_CUDA_TRY(cudaMemcpyAsync(sig.data(), dsig, nb * 8, cudaMemcpyDeviceToHost, st));
    for (int b = 0; b < nb; ++b)
      if (work[b]->f_out)
        QG_CUDA_TRY(cudaMemcpyAsync(work[b]->f_out, dx + (size_t)b * N, N * 16, cudaMemcpyDeviceToHost, st));
    QG_CUDA_TRY(cudaStreamSynchronize(st));
    for (int b = 0; b < nb; ++b) {
      work[b]->res.sigma_ext = sig[b];
      work[b]->res.residual = res[b];
      work[b]->res.iters = its[b];
      work[b]->res.fallback = fb[b];
      if (info[b]) {
        work[b]->res.status = QPMS_ERROR;
        work[b]->err = "singular matrix";
      }
    }
    return QPMS_SUCCESS;
  }

  // plane-wave incidence of a request: finite systems use its direction and
  // polarisation; periodic ones the in-plane wavevector k with x polarisation
  // projected perpendicular to the wavevector (as the dispersion scan does)
  static int incidence(const Job *j, qg_c k, int lMax, double kvec[3], std::vector<qg_c> &coef) {
    const double kap = k.re;
    if (!j->periodic) {
      const double *kd = j->req.k_dir;
      const double kn = sqrt(kd[0] * kd[0] + kd[1] * kd[1] + kd[2] * kd[2]);
      if (kn == 0) {
        set_error("zero incidence direction");
        return QPMS_EINVAL;
      }
      for (int c = 0; c < 3; ++c) kvec[c] = kap * kd[c] / kn;
      planewave_direction_coeffs(lMax, kd, j->req.E, coef);
      return QPMS_SUCCESS;
    }
    const double bx = j->req.k[0], by = j->req.k[1], b2 = bx * bx + by * by;
    const bool prop = kap * kap > b2;
    const double kz = prop ? sqrt(kap * kap - b2) : 0.0;
    const double kd[3] = {bx, by, kz};
    const double kn = sqrt(b2 + kz * kz);
    double E[3] = {1, 0, 0};
    if (kn > 0)
      for (int c = 0; c < 3; ++c) E[c] -= (kd[0] / kn) * kd[c] / kn;
    const double En = sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
    qpms_complex_t Ec[3];
    for (int c = 0; c < 3; ++c) {
      Ec[c].re = En > 0 ? E[c] / En : 0;
      Ec[c].im = 0;
    }
    const double kdd[3] = {bx, by, prop ? kz : 1.0};
    planewave_direction_coeffs(lMax, kdd, Ec, coef);
    if (!prop)
      for (auto &c : coef) c = cmk(0, 0);
    for (int c = 0; c < 3; ++c) kvec[c] = kd[c];
    return QPMS_SUCCESS;
  }

  // M = I - T S (finite) or I - T W (periodic, paired (omega, k) list), row-major
  int assemble(bool periodic, const qpms_scatsys_t *ss, int nb, const SysDev &sd, const qg_c *dT, const qg_c *dk,
               const qpms_gpu_request_t *one, const qg_c *k_one, double *dbeta, double *deta, int *derr, qg_c *dM,
               cudaStream_t st) {
    if (!periodic) {
      AsmArgs a;
      a.nw = nb;
      a.np = ss->p_count;
      a.ntm = ss->tm_count;
      a.dense = scatsys_dense(ss) ? 1 : 0;
      a.J = QPMS_HANKEL_PLUS;
      a.pos = sd.pos;
      a.tmid = sd.tmid;
      a.T = dT;
      a.k = dk;
      a.M = dM;
      return launch_assemble(a, priv(ss->c)->dev, st);
    }
    if (one) {  // single periodic request: beta / eta not uploaded yet
      const double kk[3] = {one->k[0], one->k[1], 0.0};
      qpms_complex_t kc;
      kc.re = k_one->re;
      kc.im = k_one->im;
      const double eta = qpms_ss_adjusted_eta(ss, kc, kk);
      QG_CUDA_TRY(cudaMemcpyAsync(dbeta, kk, 16, cudaMemcpyHostToDevice, st));
      QG_CUDA_TRY(cudaMemcpyAsync(deta, &eta, 8, cudaMemcpyHostToDevice, st));
      QG_CUDA_TRY(cudaStreamSynchronize(st));  // kk, eta are locals
    }
    EwaldArgs a;
    a.nw = nb;
    a.nk = 1;
    a.paired = 1;
    a.np = ss->p_count;
    a.ntm = ss->tm_count;
    a.pos = sd.pos;
    a.tmid = sd.tmid;
    a.T = dT;
    a.k = dk;
    a.beta = dbeta;
    a.eta = deta;
    a.M = dM;
    a.err = derr;
    a.layered = layered_system(ss);
    if (scatsys_dense(ss)) return ewald_assemble_dense(ss, a, (int)(ss->fecv_size / ss->p_count), st);
    return ewald_assemble_locked(ss, a, st);
  }
};

extern "C" {

qpms_gpu_server_t *qpms_gpu_server_create(size_t hbm_budget_bytes, int mode, int workers) {
  clear_error();
  if (mode != 0 && mode != 1) {
    set_error("mode must be 0 (FP64) or 1 (mixed)");
    return nullptr;
  }
  qpms_gpu_server *s = new (std::nothrow) qpms_gpu_server();
  if (!s) {
    set_error("out of host memory");
    return nullptr;
  }
  s->mode = mode;
  s->nworkers = workers > 0 ? std::min(workers, 16) : 4;
  if (cudaGetDevice(&s->device) != cudaSuccess) {
    set_error("no CUDA device");
    delete s;
    return nullptr;
  }
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    set_error("cudaMemGetInfo failed");
    delete s;
    return nullptr;
  }
  s->budget = hbm_budget_bytes ? std::min(hbm_budget_bytes, fr) : (size_t)(0.6 * fr);
  cudaMemPoolProps props;
  memset(&props, 0, sizeof props);
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = s->device;
  if (cudaMemPoolCreate(&s->pool, &props) != cudaSuccess) {
    set_error("cudaMemPoolCreate failed");
    delete s;
    return nullptr;
  }
  uint64_t keep = UINT64_MAX;  // freed blocks stay in the pool for the next request
  cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  s->t0 = std::chrono::steady_clock::now();
  for (int i = 0; i < s->nworkers; ++i) s->workers.emplace_back([s] { s->worker_main(); });
  return s;
}

int qpms_gpu_server_submit(qpms_gpu_server_t *s, const qpms_gpu_request_t *req, qpms_complex_t *f_out,
                           uint64_t *ticket) {
  clear_error();
  if (!s || !req || !req->ss || !ticket) {
    set_error("NULL argument");
    return QPMS_EINVAL;
  }
  const qpms_scatsys_t *ss = req->ss;
  if (!scatsys_is_own(ss) || (ss->lattice_dimension != 0 && ss->lattice_dimension != 2)) {
    set_error("request system must come from qpms_gpu_scatsys_create_spheres[_2d]");
    return QPMS_EINVAL;
  }
  if (!(req->omega > 0)) {
    set_error("omega must be positive");
    return QPMS_EINVAL;
  }
  Job *j = new (std::nothrow) Job();
  if (!j) {
    set_error("out of host memory");
    return QPMS_ENOMEM;
  }
  j->req = *req;
  j->f_out = f_out;
  j->N = ss->fecv_size;
  j->periodic = ss->lattice_dimension == 2;
  j->small = j->N <= kSmallN;
  j->bytes = s->job_bytes(*j);
  memset(&j->res, 0, sizeof j->res);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (j->bytes > s->budget) {
      delete j;
      set_error("request needs %zu device bytes, above the server budget %zu", j->bytes, s->budget);
      return QPMS_ENOMEM;
    }
    j->id = s->next_id++;
    j->res.t_submit = s->now();
    s->jobs[j->id] = j;
    s->pending.push_back(j);
    *ticket = j->id;
  }
  s->cv_work.notify_one();
  return QPMS_SUCCESS;
}

int qpms_gpu_server_wait(qpms_gpu_server_t *s, uint64_t ticket, qpms_gpu_result_t *out) {
  clear_error();
  if (!s) return QPMS_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) {
    set_error("unknown ticket %llu", (unsigned long long)ticket);
    return QPMS_EINVAL;
  }
  Job *j = it->second;
  s->cv_done.wait(lk, [&] { return j->done; });
  if (out) *out = j->res;
  const int st = j->res.status;
  if (st) set_error("%s", j->err.c_str());
  s->jobs.erase(it);
  delete j;
  return st;
}

int qpms_gpu_server_cancel(qpms_gpu_server_t *s, uint64_t ticket) {
  clear_error();
  if (!s) return QPMS_EINVAL;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) {
      set_error("unknown ticket %llu", (unsigned long long)ticket);
      return QPMS_EINVAL;
    }
    Job *j = it->second;
    auto q = std::find(s->pending.begin(), s->pending.end(), j);
    if (q == s->pending.end()) {
      set_error("request %llu has already started", (unsigned long long)ticket);
      return QPMS_EINVAL;
    }
    s->pending.erase(q);
    j->res.status = QPMS_ECANCELED;
    j->res.t_start = j->res.t_done = s->now();
    j->err = "cancelled before it started";
    j->done = true;
  }
  s->cv_done.notify_all();
  s->cv_work.notify_all();
  return QPMS_SUCCESS;
}

int qpms_gpu_server_testing_fail_allocations(qpms_gpu_server_t *s, int count) {
  if (!s || count < 0) return QPMS_EINVAL;
  g_fail_allocs.store(count);
  return QPMS_SUCCESS;
}

int qpms_gpu_server_drain(qpms_gpu_server_t *s) {
  if (!s) return QPMS_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_done.wait(lk, [&] { return s->pending.empty() && s->busy == 0; });
  return QPMS_SUCCESS;
}

double qpms_gpu_server_clock(qpms_gpu_server_t *s) { return s ? s->now() : 0.0; }

int qpms_gpu_server_stats(qpms_gpu_server_t *s, size_t *completed, size_t *batches, size_t *peak_bytes,
                          int *max_concurrent, size_t *budget_bytes) {
  if (!s) return QPMS_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  if (completed) *completed = s->completed;
  if (batches) *batches = s->batches;
  if (peak_bytes) *peak_bytes = s->peak;
  if (max_concurrent) *max_concurrent = s->max_busy;
  if (budget_bytes) *budget_bytes = s->budget;
  return QPMS_SUCCESS;
}

void qpms_gpu_server_destroy(qpms_gpu_server_t *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto &t : s->workers) t.join();
  cudaSetDevice(s->device);
  for (void *p : s->sys_ptrs) cudaFreeAsync(p, 0);
  cudaStreamSynchronize(0);
  for (auto &kv : s->jobs) delete kv.second;
  for (Job *j : s->pending)
    if (s->jobs.find(j->id) == s->jobs.end()) delete j;
  if (s->pool) cudaMemPoolDestroy(s->pool);
  delete s;
}

}  // extern "C"
