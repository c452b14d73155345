// Device-side pieces of the mode-problem pipeline (qg_assembly.cu).
#pragma once
#include <cuda_runtime.h>

#include "qg_internal.h"

namespace qg {

// Arguments of the batched assembly kernel.
struct AsmArgs {
  int nw;             // frequencies (matrices) in the batch
  int np;             // particles
  int ntm;            // T-matrix types
  int dense;          // 0: T stored as diagonals [nw][ntm][n]; 1: dense [nw][ntm][n][n]
  int J;              // Bessel kind of S (3 = Hankel+ for M = I - T S)
  const double *pos;  // [np][3]
  const int *tmid;    // [np]
  const qg_c *T;      // T-matrices per (w, type)
  const qg_c *k;      // [nw] medium wavenumbers
  qg_c *M;            // [nw][N][N], N = np * 2 nelem, row-major
};

int launch_assemble(const AsmArgs &a, const TransDevTables &T, cudaStream_t st);
// a[w][p n + i] = coef[w coef_stride + i] exp(i kvec_w . r_p)
int launch_incident(int nw, int np, int n, const qg_c *coef, const double *kvec, const double *pos, qg_c *a,
                    cudaStream_t st, size_t coef_stride = 0);
int launch_apply_t(int nw, int np, int n, int ntm, int dense, const int *tmid, const qg_c *T, const qg_c *a,
                   qg_c *b, cudaStream_t st);
int launch_residual(int nw, size_t N, const qg_c *M, const qg_c *x, const qg_c *b, qg_c *r, double *rn2,
                    double *bn2, cudaStream_t st);
int launch_c128_to_c64(size_t n, const qg_c *src, void *dst, cudaStream_t st);
int launch_add_c64(size_t n, const void *dx, qg_c *x, int init, cudaStream_t st);
int launch_sigma_ext(int nw, size_t N, const qg_c *a, const qg_c *f, const qg_c *k, double *sig, cudaStream_t st);
int launch_transpose(size_t n, int nb, const qg_c *src, qg_c *dst, cudaStream_t st);

}  // namespace qg
