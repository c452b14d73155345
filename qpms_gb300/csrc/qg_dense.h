// Large dense complex solver (qg_dense.cu): RBT + blocked LU without pivoting,
// complex64 (mixed, FP64 iterative refinement) or complex128 (plain).
#pragma once
#include <cuda_runtime.h>

#include "qg_ozaki.h"

namespace qg {

// Right-hand-side count from which the refinement residual runs as digit
// products on the bf16 tensor cores (qg_ozaki.cu) instead of a complex128
// GEMM; below it the residual is bandwidth-bound on M and the FP64 GEMM is
// cheaper.  QPMS_GB300_RESIDUAL=ZGEMM turns the digit path off.
constexpr int kOzakiMinRhs = 8;
// Largest group of blocks of the tensor-core LU (DenseSolver::group).
constexpr int kMaxLuGroup = 4;
bool ozaki_wanted(int nrhs_max);
// Whether a solver for many right-hand sides keeps the digit planes of its
// factors (QPMS_GB300_FACTOR_PLANES=0 turns it off).
bool fac_planes_wanted();

// The system is padded to Np = N rounded up to a multiple of 4 (identity on the
// padding), the size the two butterfly levels halve.
struct DenseSolver {
  int N = 0, Np = 0, nrhs_max = 0, mode = 0, nb = 64;
  void *A = nullptr;       // mode 1: complex64 LU factors, Np x Np (mode 0 factors T64 in place)
  void *T64 = nullptr;     // complex128 Np x Np: W_u^T diag(M, I) W_v (mode 0; mode 1 at its first fallback)
  void *Dinv = nullptr;    // per diagonal block: L^-1 and U^-1 (nb x nb each)
  void *work = nullptr;    // panel / RHS work buffer
  void *rhs_lo = nullptr;  // complex64 Np x nrhs_max
  void *rp = nullptr;      // complex128 Np x nrhs_max (padded right-hand sides)
  void *r64 = nullptr, *y64 = nullptr;  // complex128 N x nrhs_max: residual and correction
  int *dinfo = nullptr;    // zero-pivot flag, then two doubles of norm scratch
  double *rs = nullptr;    // butterfly diagonals [u L1][u L2][v L1][v L2], Np each
  double *res_nrm = nullptr;  // norms scratch of the few-right-hand-side residual kernel
  unsigned *sweep = nullptr;  // sync words of the one-launch substitution sweeps (error word first)

  // Stream-ordered allocation: with a memory pool, every buffer comes from
  // cudaMallocFromPoolAsync on stream `ast` and returns to it in release(),
  // so a serving loop allocates without synchronising the device.
  cudaMemPool_t pool = nullptr;
  cudaStream_t ast = nullptr;
  bool row_major = false;  // set by factorize(): M64 is row-major (the reference's layout)
  int trail_ct = 0;        // cublasComputeType_t of the complex64 trailing updates (mode 1, tc_split 0)
  int tc_split = 0;        // mode 1 on the tensor cores: bf16 digits per operand (2 or 3); 0: cuBLAS
  int base_tc = 0;
  void *tc_pa = nullptr, *tc_pb = nullptr;  // digit planes of the GEMM operands
  void *fac_planes = nullptr;  // 3-digit planes of the whole factored matrix (many right-hand sides)
  int refactors = 0;       // refinement stalls answered by more precise factors
  int base_mode = 0, base_trail = 0;  // what factorize() starts from (the fallbacks change mode / trail_ct)
  // digit slices of M for the tensor-core residual (nrhs_max >= kOzakiMinRhs)
  bool use_ozaki = false;
  void *oz_mat = nullptr, *oz_work = nullptr;
  OzakiMatrix oz;

  // CUDA graphs for solvers that repeat the same launch sequence on the same
  // buffers (the Beyn contour nodes): with `graphs` set (and the environment
  // variable QPMS_GB300_GRAPHS not 0), factorize() and apply_inverse() run
  // eagerly at the first call with a given set of buffers, are captured on
  // the second and replayed from then on.  Only the mixed tensor-core and
  // few-right-hand-side paths are captured, on streams other than the legacy
  // default stream, and not while per-launch timing is on.
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    unsigned long long key[6] = {0, 0, 0, 0, 0, 0};
    bool keyed = false;
    unsigned long long launches = 0;  // kernel launches of one replay
  };
  bool graphs = false;
  Graph gf, gs;
  // lookahead of the tensor-core LU: the next diagonal block is inverted on
  // `side` (high priority) while the trailing update runs (QPMS_GB300_LOOKAHEAD=0
  // turns it off; so does lookahead = false before init(): a serving loop with
  // several workers already overlaps the inversions with other requests' work)
  bool lookahead = true;
  // few-right-hand-side substitutions as one launch per sweep (tiles that wait
  // on per-block counters) rather than one launch per block and sweep; a
  // serving loop with several workers turns it off: the waiting CTAs would hold
  // SMs that other requests' GEMMs need (QPMS_GB300_SUBST=sweep / steps
  // overrides either way)
  bool sweeps = true;
  // tensor-core LU by groups of `group` blocks (1 .. kMaxLuGroup): one
  // trailing update with K = group x nb per group (QPMS_GB300_LU_GROUP
  // overrides); set before init(), which sizes the operand planes for it
  int group = 2;
  // block size of the complex64 LU: 0 = the tuned choice (lu_block_size), else
  // 64 or 128; set before init()
  int nb_pref = 0;
  cudaStream_t side = nullptr;
  cudaEvent_t ev_a = nullptr, ev_d = nullptr;
  unsigned long long graph_replays = 0;

  int init(int N, int nrhs_max, int mode, unsigned long long seed, cudaMemPool_t pool = nullptr,
           cudaStream_t alloc_stream = nullptr);
  void release();
  ~DenseSolver() { release(); }
  // M64: device complex128 N x N with leading dimension ldm, column-major, or
  // row-major if rowmaj (kept by the caller: the refinement residual is formed
  // with it).
  int factorize(const void *M64, size_t ldm, cudaStream_t st, bool rowmaj = false);
  int factorize_current(const void *M64, size_t ldm, cudaStream_t st);  // with the current mode / trail_ct
  // Y = M^-1 R through the factors (one application, no refinement); N x nrhs.
  int apply_inverse(const void *R, size_t ldr, void *Y, size_t ldy, int nrhs, cudaStream_t st);
  // X = M^-1 B (B, X: N x nrhs, leading dimension N), refined with FP64
  // residuals until ||B - M X||_F / ||B||_F <= tol, stagnation or max_iter.
  // resid_out gets the final FP64 relative residual, iters_out the number of
  // applications of the factors.
  int solve(const void *M64, size_t ldm, const void *B, void *X, int nrhs, double tol, int max_iter,
            double *resid_out, int *iters_out, cudaStream_t st);
  // Device bytes init() allocates for (N, nrhs, mode).
  static size_t footprint(int N, int nrhs, int mode);

 private:
  cudaError_t dev_alloc(void *ptr, size_t bytes);
  int check_info(cudaStream_t st);  // zero-pivot flag of the last factorisation
  bool use_sweeps() const;
  int lu_group() const;
  int factor_launch(const void *M64, size_t ldm, cudaStream_t st);  // factorize_current's launches
  int apply_launch(const void *R, size_t ldr, void *Y, size_t ldy, int nrhs, cudaStream_t st);
  template <class F>
  int run_graph(Graph &g, const unsigned long long (&key)[6], bool capturable, cudaStream_t st, F body);
};

}  // namespace qg
