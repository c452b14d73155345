// Small dense complex linear algebra on the host for the Beyn eigensolver's
// post-processing (m x L with L <= a few hundred, and L x L): thin SVD and the
// general eigenproblem.  Column-major storage, A(i, j) = A[i + j * lda].
#pragma once
#include <complex>
#include <cstddef>

namespace qg {
namespace hostla {

typedef std::complex<double> cd;

// Thin SVD A = U diag(s) V^H of an m x n matrix, m >= n (the reference's
// LAPACKE_zgesdd with jobz 'O', beyn.c:321-333): Householder QR, then
// one-sided Jacobi on R.  s is descending; U is m x n, V is n x n.
// Returns 0, or -1 if the Jacobi sweeps do not converge.
int svd_thin(int m, int n, const cd *A, int lda, cd *U, double *s, cd *V);

// Eigenvalues w and right eigenvectors X (n x n, column k for w[k]) of a
// general complex matrix (the reference's LAPACKE_zgeev with jobvr 'V',
// beyn.c:404-416): Householder Hessenberg reduction, single-shift complex QR
// with Wilkinson shifts, back substitution on the Schur form.  Each vector
// has unit 2-norm and its largest component real, as zgeev returns them.
// Returns 0, or -1 if the QR iteration does not converge.
int eig(int n, const cd *A, int lda, cd *w, cd *X);

// Complex Gaussian probe matrix (real and imaginary parts N(0, 1), as
// zrandN(1, 0) in beyn.c:46-56) from a seeded splitmix64 stream; row-major
// m x l (the layout of the reference's VHat).
void probe_matrix(size_t m, size_t l, unsigned long long seed, cd *out);

}  // namespace hostla
}  // namespace qg
