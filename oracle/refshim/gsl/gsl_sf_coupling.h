/* Minimal stand-in for GSL's gsl_sf_coupling.h (oracle test infrastructure). */
#ifndef QG_REFSHIM_GSL_SF_COUPLING_H
#define QG_REFSHIM_GSL_SF_COUPLING_H
double gsl_sf_coupling_3j(int two_ja, int two_jb, int two_jc, int two_ma, int two_mb, int two_mc);
#endif
