/* Stand-in declaration of the Faddeeva package's w(z) (S. G. Johnson's MIT
 * library, not vendored with the reference).  The reference's ewaldsf.c calls
 * it only for the Kambe sums of layers at different heights, which the oracle
 * does not compare through the reference's own code; the stand-in returns NaN.
 * Oracle test infrastructure. */
#ifndef QG_REFSHIM_FADDEEVA_H
#define QG_REFSHIM_FADDEEVA_H
#include <complex.h>
double complex Faddeeva_w(double complex z, double relerr);
#endif
