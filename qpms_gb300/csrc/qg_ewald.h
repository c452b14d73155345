// Device-side Ewald lattice sums (qg_ewald.cu).
#pragma once
#include <cuda_runtime.h>

#include "qg_internal.h"

namespace qg {

// Largest sigma order lMax_e = 2 lMax + 1 compiled (lMax <= 4).
constexpr int kEwLE = 9;
constexpr int kEwS = (kEwLE + 1) * (kEwLE + 1);
// Number of (n, m, j, s) terms of the shifted long-range sum at lMax_e = kEwLE.
constexpr int kEwZ = 420;

// Lattice- and convention-dependent constants (one lattice at a time).
struct EwaldConst {
  double b[4];    // direct basis b1 (x, y), b2 (x, y)
  double rb[4];   // reciprocal basis (2 pi normalised)
  double bn[2];   // |b1|, |b2|
  double rbn[2];  // |rb1|, |rb2|
  double area;    // unit cell area
  // P_n^{|m|}(0) (-1)^{m<0 ? m : 0} per y = n(n+1) + m (ewald.c:425, 877, 886)
  double leg0m[kEwS];
  // long-range constants s1_constfacs[y][j] (ewald.c:142-146) times leg0m[y],
  // and the same as s1 = i^(n+1) s1r with s1r real
  int s1off[kEwS];
  qg_c s1[kEwS * (kEwLE / 2 + 1)];
  double s1r[kEwS * (kEwLE / 2 + 1)];
  // Pairs of layers at different heights (shift.z != 0):
  // sign factors of leg_nm(x) = legs[y] P_n^|m|(x) with the Condon-Shortley
  // phase in P (m1pow_m_neg(m), and (-1)^m for csphase +1)
  double legs[kEwS];
  // long-range constants S1[y][j, s] (derived for the shifted sum; entries
  // zoff[y] .. zoff[y + 1] - 1 in (j, s) order) with their j and s
  int zoff[kEwS + 1];
  qg_c zs1[kEwZ];
  unsigned char zj[kEwZ], zsv[kEwZ];
};

struct EwaldArgs {
  int nw, nk, np, ntm;
  const double *pos;   // [np][3]
  const int *tmid;     // [np]
  const qg_c *T;       // [nw][ntm][n] diagonal T-matrices
  const qg_c *k;       // [nw] medium wavenumbers
  const double *beta;  // [nk][2] Bloch vectors
  const double *eta;   // [nw * nk] Ewald parameters
  qg_c *M;             // [nw * nk][N][N]
  int *err;            // bit 1: a unit's lattice-point range exceeded the bound
  int paired = 0;      // 1: nk == 1 and matrix w uses Bloch vector beta[w] (a list of (omega, k) pairs)
  // Optional list of particle pairs (R, C): only those blocks are formed,
  // block p of matrix wk at M + (wk * npairs + p) * NB * NB (row-major NB x NB)
  // instead of the full N x N matrices.
  int npairs = 0;
  const int *pairs = nullptr;  // [npairs][2]
  // 1: some pair lies in different planes (z_R != z_C); those blocks are
  // formed by a second kernel.  A pair with z_R != z_C and layered == 0 sets
  // bit 2 of *err.
  int layered = 0;
  // Short-range tables (dispersion scans, not with `paired`): when srtab is
  // set, eta[w * nk + k] must be one value per frequency w, and the
  // single-plane kernel takes the short-range terms c_nm(R) of (w, pair) from
  // the tables (formed once per (w, pair) by the table kernel) and applies
  // only the Bloch phase e^{i beta.(R - s)}: the radial integrals do not
  // depend on beta.
  qg_c *srtab = nullptr;   // [nw][pairs][NEVEN][srmax]
  double *srpts = nullptr; // [nw][pairs][srmax][2]: R - s in the plane
  int *srcnt = nullptr;    // [nw][pairs]
  int srmax = 0;
};

// Bound on the lattice points one unit may enumerate per sum.
constexpr long kEwMaxPoints = 1L << 22;

int ewald_upload_constants(const EwaldConst &c, cudaStream_t st);
int launch_ewald_assemble(const EwaldArgs &a, const TransDevTables &T, cudaStream_t st);

}  // namespace qg
