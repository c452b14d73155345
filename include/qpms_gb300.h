/*
 * libqpms_gb300 -- GB300 (sm_103a) implementation of the QPMS mode-problem hot
 * path behind the reference's own C API.
 *
 * Conventions kept from the reference (kostyfisik/qpms):
 *   - complex numbers are `complex double` (two doubles, re then im);
 *   - matrices are row-major C order, strides counted in elements (translations.h:14-17);
 *   - functions return 0 (QPMS_SUCCESS) or a non-zero qpms_errno_t-style code;
 *   - VSWF index y = n(n+1) + m - 1 (indexing.h:13-15), nelem = lMax(lMax+2).
 * Additions: qpms_gpu_* batched entry points over device pointers, and
 * qpms_gpu_last_error() for a thread-local error message.  The library never
 * aborts; every CUDA failure becomes a non-zero return code.
 */
#ifndef QPMS_GB300_H
#define QPMS_GB300_H

#include <stddef.h>
#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
typedef struct { double re, im; } qpms_complex_t;
#else
#include <complex.h>
typedef double complex qpms_complex_t;
#endif

/* ---------------- types (qpms_types.h of the reference) ---------------- */
typedef int qpms_l_t;                 /* qpms_types.h:27 */
typedef int qpms_m_t;                 /* qpms_types.h:31 */
typedef size_t qpms_y_t;              /* qpms_types.h:44 */
typedef int qpms_normalisation_t;     /* enum, qpms_types.h:104-168 */
typedef int qpms_bessel_t;            /* enum, qpms_types.h:176-182: 1 j, 2 y, 3 h+, 4 h- */

#define QPMS_SUCCESS 0
#define QPMS_ERROR 1
#define QPMS_ENOMEM 12
#define QPMS_EINVAL 22
#define QPMS_ECANCELED 125
#define QPMS_NAN_ENCOUNTERED 1024  /* qpms_types.h:91 */
#define QPMS_NORMALISATION_INVERSE 1
#define QPMS_NORMALISATION_REVERSE_AZIMUTHAL_PHASE 2
#define QPMS_NORMALISATION_SPHARM_REAL 4
#define QPMS_NORMALISATION_CSPHASE 8
#define QPMS_NORMALISATION_M_I 16
#define QPMS_NORMALISATION_M_MINUS 32
#define QPMS_NORMALISATION_N_I 64
#define QPMS_NORMALISATION_N_MINUS 128
#define QPMS_NORMALISATION_NORM_POWER 65536
#define QPMS_NORMALISATION_NORM_NONE (65536 * 2)
#define QPMS_NORMALISATION_NORM_SPHARM (65536 * 3)
#define QPMS_NORMALISATION_DEFAULT (QPMS_NORMALISATION_NORM_POWER | QPMS_NORMALISATION_CSPHASE)
#define QPMS_BESSEL_REGULAR 1
#define QPMS_BESSEL_SINGULAR 2
#define QPMS_HANKEL_PLUS 3
#define QPMS_HANKEL_MINUS 4

/* Spherical coordinates with complex radial part, qpms_types.h:212-216. */
typedef struct csph_t {
  qpms_complex_t r;
  double theta, phi;
} csph_t;

/* Translation calculator, same field order as translations.h:64-84 (built
 * with LATTICESUMS32, so e3c is present).  The multiplier tables are the
 * reference's ragged host tables; the device copies live in a private
 * extension that follows this struct in memory. */
typedef struct qpms_trans_calculator {
  qpms_normalisation_t normalisation;
  qpms_l_t lMax;
  qpms_y_t nelem;
  qpms_complex_t **A_multipliers;
  qpms_complex_t **B_multipliers;
  void *e3c;
  double *legendre0;
} qpms_trans_calculator;

/* ---------------- translation operator ---------------- */

/* Replaces qpms_trans_calculator_init (translations.h:87-89, translations.c:439-508).
 * Builds the A/B multiplier tables on the host and uploads the kernel's tables
 * to the current CUDA device.  Returns NULL on error (see qpms_gpu_last_error). */
qpms_trans_calculator *qpms_trans_calculator_init(qpms_l_t lMax, qpms_normalisation_t nt);

/* Replaces qpms_trans_calculator_free (translations.h:91, translations.c:288-298). */
void qpms_trans_calculator_free(qpms_trans_calculator *c);

/* Replaces qpms_trans_calculator_get_AB_arrays (translations.h:103-106,
 * translations.c:688-698): one translation kdlj, host output buffers
 * A[deststride*y + srcstride*yu], B likewise; computed on the GPU. */
int qpms_trans_calculator_get_AB_arrays(const qpms_trans_calculator *c,
    qpms_complex_t *Adest, qpms_complex_t *Bdest,
    size_t deststride, size_t srcstride,
    csph_t kdlj, bool r_ge_d, qpms_bessel_t J);

/* Replaces qpms_trans_calculator_get_AB_arrays_ext (translations.h:122-126,
 * translations.c:1124-1132), the variant the Cython wrapper binds. */
int qpms_trans_calculator_get_AB_arrays_ext(const qpms_trans_calculator *c,
    qpms_complex_t *Adest, qpms_complex_t *Bdest,
    size_t deststride, size_t srcstride,
    qpms_complex_t kdlj_r, double kdlj_theta, double kdlj_phi,
    int r_ge_d, int J);

/* Batched translation coefficients on DEVICE pointers (the batched form of
 * the numpy loop qpms_cython_trans_calculator_get_AB_arrays_loop,
 * translations_python.c:24-132, which binds trans_calculator.get_AB_arrays,
 * cytranslations.pyx:405-512; extended to complex kr as in the C API).
 * For i < n: kd_i = (kr[i], theta[i], phi[i]); r_ge_d may be NULL (all false).
 * Output A[i][y][yu], B[i][y][yu], complex128, 16-byte aligned.
 * stream: a cudaStream_t (NULL = legacy default stream).  Asynchronous. */
int qpms_gpu_trans_AB_arrays_batch(const qpms_trans_calculator *c, size_t n,
    const qpms_complex_t *kr, const double *theta, const double *phi,
    const unsigned char *r_ge_d, qpms_bessel_t J,
    qpms_complex_t *A, qpms_complex_t *B, void *stream);

/* Same on HOST pointers: pinned staging, chunked and pipelined over two
 * streams (host->device copy, kernel, device->host copy overlap).
 * Synchronous.  This is what the Python trans_calculator.get_AB_arrays calls. */
int qpms_gpu_trans_AB_arrays_batch_host(const qpms_trans_calculator *c, size_t n,
    const qpms_complex_t *kr, const double *theta, const double *phi,
    const unsigned char *r_ge_d, qpms_bessel_t J,
    qpms_complex_t *A, qpms_complex_t *B);

/* Allocation-free form of qpms_gpu_trans_AB_arrays_batch_host, for callers
 * that must not allocate device or pinned memory while they run (a process
 * whose device memory is owned by a pool allocator or capped by a budget, a
 * real-time loop that forbids allocation after start-up, a plug-in that must
 * not change its host's memory footprint).  No counterpart in the reference.
 * Same kernel and results; inputs and outputs are host buffers.  Staging uses
 * a file-scope device array of 32 MiB that every GPU loading the library holds
 * until exit, so a batch must fit in it (about 4,600 translations at lMax 3,
 * 450 at lMax 6); larger batches are rejected with QPMS_EINVAL and a message.
 * The first call on a device looks up the array's device address (once per
 * device, with that device current); make that first call before any stream
 * capture.  All calls share the array and it keeps the last call's contents;
 * calls that overlap on the GPU race on it, so serialise them.  Synchronous,
 * on the legacy default stream. */
int qpms_gpu_trans_AB_arrays_batch_host_noalloc(const qpms_trans_calculator *c, size_t n,
    const qpms_complex_t *kr, const double *theta, const double *phi,
    const unsigned char *r_ge_d, qpms_bessel_t J,
    qpms_complex_t *A, qpms_complex_t *B);

/* Every entry point that takes a calculator checks that the current device is
 * the one current at qpms_trans_calculator_init (its device tables live
 * there) and returns QPMS_EINVAL otherwise.  Test hook: overwrites the device
 * recorded in the calculator, so that tests on a one-GPU machine can provoke
 * that mismatch; no counterpart in the reference, not for production use. */
int qpms_gpu_testing_set_calculator_device(qpms_trans_calculator *c, int device);

/* Number of A / B multipliers (ragged table sizes), for tests. */
size_t qpms_gpu_trans_calculator_n_multipliers(const qpms_trans_calculator *c, int which_B);

/* Host-only export of the ragged A/B multiplier tables of
 * qpms_trans_calculator_init (same order as the reference's
 * A_multipliers[0][...], translations.c:464-471), computed without a GPU.
 * *nA, *nB: capacity on input, table size on output; NULL outputs query sizes. */
int qpms_gpu_trans_multipliers_export(qpms_l_t lMax, qpms_normalisation_t nt,
    qpms_complex_t *A_out, size_t *nA, qpms_complex_t *B_out, size_t *nB);


/* ---------------- scattering systems (scatsystem.h of the reference) ----------------
 * Struct layouts are field-for-field those of the reference (qpms_types.h,
 * scatsystem.h, materials.h), so objects built by the reference's own
 * constructors can be passed to the drop-in functions below.  Members the hot
 * path never reads (symmetry orbits, irrep bases, generator tables) are kept as
 * opaque pointers of the same size. */
typedef struct cart3_t { double x, y, z; } cart3_t;                 /* qpms_types.h:186-189 */
typedef struct cart2_t { double x, y; } cart2_t;                     /* qpms_types.h:202-204 */
typedef struct ccart3_t { qpms_complex_t x, y, z; } ccart3_t;        /* qpms_types.h:192-195 */
typedef unsigned long long qpms_uvswfi_t;                            /* qpms_types.h:81 */
typedef int qpms_iri_t;                                              /* qpms_types.h:323 */
typedef int32_t qpms_ss_tmi_t, qpms_ss_tmgi_t, qpms_ss_pi_t;         /* qpms_types.h:310-316 */

typedef struct qpms_vswf_set_spec_t {                                /* qpms_types.h:290-308 */
  size_t n;
  qpms_uvswfi_t *ilist;
  qpms_l_t lMax, lMax_M, lMax_N, lMax_L;
  size_t capacity;
  qpms_normalisation_t norm;
} qpms_vswf_set_spec_t;

/* Replaces qpms_trans_calculator_get_trans_array (translations.h:129-135,
 * translations.c:701-722): the translation operator between two VSWF sets
 * (same normalisation as c, lMax <= c->lMax, no longitudinal waves) for one
 * displacement kdlj, target[srci * srcstride + desti * deststride] = A or B
 * (translations_inlines.h:8-35); computed on the GPU. */
int qpms_trans_calculator_get_trans_array(const qpms_trans_calculator *c, qpms_complex_t *target,
    const qpms_vswf_set_spec_t *destspec, size_t deststride,
    const qpms_vswf_set_spec_t *srcspec, size_t srcstride,
    csph_t kdlj, bool r_ge_d, qpms_bessel_t J);

/* Replaces qpms_trans_calculator_get_trans_array_lc3p (translations.h:139-149,
 * translations.c:796-812): the same from wavenumber k and cartesian positions,
 * kdlj = k * (destpos - srcpos) in spherical coordinates, r_ge_d = false. */
int qpms_trans_calculator_get_trans_array_lc3p(const qpms_trans_calculator *c, qpms_complex_t *target,
    const qpms_vswf_set_spec_t *destspec, size_t deststride,
    const qpms_vswf_set_spec_t *srcspec, size_t srcstride,
    qpms_complex_t k, cart3_t destpos, cart3_t srcpos, qpms_bessel_t J);

typedef struct qpms_tmatrix_t {                                      /* qpms_types.h:338-351 */
  const qpms_vswf_set_spec_t *spec;
  qpms_complex_t *m;  /* row-major spec->n x spec->n */
  bool owns_m;
} qpms_tmatrix_t;

typedef struct qpms_epsmu_t { qpms_complex_t eps, mu; } qpms_epsmu_t; /* qpms_types.h:422-425 */

typedef struct qpms_epsmu_generator_t {                              /* materials.h:16-25 */
  qpms_epsmu_t (*function)(qpms_complex_t omega, const void *params);
  const void *params;
} qpms_epsmu_generator_t;

typedef struct qpms_particle_tid_t {                                 /* scatsystem.h:36-40 */
  cart3_t pos;
  qpms_ss_tmi_t tmatrix_id;
} qpms_particle_tid_t;

typedef struct qpms_scatsys_periodic_info_t {                        /* scatsystem.h:135-158 */
  cart3_t lattice_basis[3];
  cart3_t reciprocal_basis[3];
  double unitcell_volume;
  double eta;
} qpms_scatsys_periodic_info_t;

typedef struct qpms_scatsys_t {                                      /* scatsystem.h:169-227 */
  int lattice_dimension;
  qpms_epsmu_generator_t medium;
  void *tmg;                    /* qpms_tmatrix_function_t * */
  qpms_ss_tmgi_t tmg_count;
  void *tm;                     /* qpms_ss_derived_tmatrix_t * */
  qpms_ss_tmi_t tm_count;
  qpms_ss_tmi_t tm_capacity;
  qpms_particle_tid_t *p;
  qpms_ss_pi_t p_count;
  qpms_ss_pi_t p_capacity;
  const void *sym;              /* const struct qpms_finite_group_t * */
  qpms_ss_pi_t *p_sym_map;
  qpms_ss_tmi_t *tm_sym_map;
  int32_t orbit_type_count;     /* qpms_ss_oti_t */
  void *orbit_types;
  void *p_orbitinfo;
  size_t fecv_size;
  size_t *saecv_sizes;
  size_t *fecv_pstarts;
  size_t *saecv_ot_offsets;
  size_t max_bspecn;
  qpms_ss_pi_t *p_by_orbit;
  char *otspace;
  char *otspace_end;
  double lenscale;
  struct qpms_trans_calculator *c;
  qpms_scatsys_periodic_info_t per;
} qpms_scatsys_t;

typedef struct qpms_scatsys_at_omega_t {                             /* scatsystem.h:239-249 */
  const qpms_scatsys_t *ss;
  qpms_tmatrix_t **tm;
  qpms_complex_t omega;
  qpms_epsmu_t medium;
  qpms_complex_t wavenumber;
} qpms_scatsys_at_omega_t;

typedef struct qpms_scatsys_at_omega_k_t {                           /* scatsystem.h:488-492 */
  const qpms_scatsys_at_omega_t *ssw;
  double k[3];
  double eta;
} qpms_scatsys_at_omega_k_t;

typedef struct qpms_ss_LU {                                          /* scatsystem.h:432-441 */
  const qpms_scatsys_at_omega_t *ssw;
  const qpms_scatsys_at_omega_k_t *sswk;
  bool full;
  qpms_iri_t iri;
  qpms_complex_t *a;
  int *ipiv;
} qpms_ss_LU;

/* -- constructors of this library (the reference builds systems through its
 *    symmetry machinery, scatsystem.c:233-604, which is outside the hot path) -- */

/* ---------------- materials (materials.h) ---------------- */
typedef struct qpms_ldparams_triple_t {                              /* materials.h:54-58 */
  double f;
  double omega;
  double gamma;
} qpms_ldparams_triple_t;

typedef struct qpms_ldparams_t {                                     /* materials.h:66-71 */
  qpms_complex_t eps_inf;
  double omega_p;
  size_t n;
  qpms_ldparams_triple_t data[];
} qpms_ldparams_t;

/* Lorentz-Drude fits of metals (materials.h:73-77; Rakic et al., Appl. Opt. 37, 5271 (1998)). */
extern const qpms_ldparams_t *const QPMS_LDPARAMS_AG;
extern const qpms_ldparams_t *const QPMS_LDPARAMS_AU;
extern const qpms_ldparams_t *const QPMS_LDPARAMS_CU;
extern const qpms_ldparams_t *const QPMS_LDPARAMS_AL;
extern const qpms_ldparams_t *const QPMS_LDPARAMS_CR;

/* materials.c:156-164: sum_j f_j omega_p^2 / (omega_j^2 - omega^2 - i omega gamma_j).
 * As in the reference, eps_inf is not added. */
qpms_complex_t qpms_lorentzdrude_eps(qpms_complex_t omega, const qpms_ldparams_t *p);

/* ---- tabulated data: interpolators (materials.h:101-145, tmatrices.h:285-330) ----
 * qpms_interp_type_t stands for the reference's gsl_interp_type: the two
 * kinds its Python layer uses, piecewise linear and the natural cubic spline
 * (gsl_interp_linear, gsl_interp_cspline).  Outside the tabulated range an
 * evaluation gives NaN. */
typedef struct qpms_interp_type_t qpms_interp_type_t;
extern const qpms_interp_type_t *const qpms_interp_linear;
extern const qpms_interp_type_t *const qpms_interp_cspline;

typedef struct qpms_permittivity_interpolator_t qpms_permittivity_interpolator_t;  /* opaque */
qpms_permittivity_interpolator_t *qpms_permittivity_interpolator_create(size_t incount,  /* materials.h:115-120 */
    const double *wavelength_m, const double *n, const double *k, const qpms_interp_type_t *iptype);
/* refractiveindex.info file, the "data: |" block of "wavelength_um n k" lines (materials.c:43-118) */
int qpms_load_refractiveindex_yml(const char *path, size_t *count, double **lambdas_m, double **n, double **k);
qpms_permittivity_interpolator_t *qpms_permittivity_interpolator_from_yml(const char *path,  /* materials.h:122-126 */
    const qpms_interp_type_t *iptype);
void qpms_permittivity_interpolator_free(qpms_permittivity_interpolator_t *interp);
qpms_complex_t qpms_permittivity_interpolator_eps_at_omega(                               /* materials.h:128-131 */
    const qpms_permittivity_interpolator_t *interp, double omega_SI);
qpms_epsmu_t qpms_permittivity_interpolator_epsmu_g(qpms_complex_t omega, const void *interp);  /* materials.h:133-139 */
qpms_epsmu_t qpms_epsmu_const_g(qpms_complex_t omega, const void *epsmu);                     /* materials.h:36-38 */
double qpms_permittivity_interpolator_omega_min(const qpms_permittivity_interpolator_t *ip);
double qpms_permittivity_interpolator_omega_max(const qpms_permittivity_interpolator_t *ip);

/* VSWF sets and T-matrices (vswf.c:76-97, tmatrices.c:56-75) */
qpms_vswf_set_spec_t *qpms_vswf_set_spec_from_lMax(qpms_l_t lMax, qpms_normalisation_t norm);
void qpms_vswf_set_spec_free(qpms_vswf_set_spec_t *s);
qpms_tmatrix_t *qpms_tmatrix_init(const qpms_vswf_set_spec_t *bspec);
void qpms_tmatrix_free(qpms_tmatrix_t *t);

typedef struct qpms_tmatrix_interpolator_t qpms_tmatrix_interpolator_t;  /* opaque; copies the basis */
qpms_tmatrix_interpolator_t *qpms_tmatrix_interpolator_create(size_t n,                 /* tmatrices.h:318-323 */
    const double *freqs, const qpms_tmatrix_t *tmatrices_array, const qpms_interp_type_t *iptype);
void qpms_tmatrix_interpolator_free(qpms_tmatrix_interpolator_t *interp);
int qpms_tmatrix_interpolator_eval_fill(qpms_tmatrix_t *target,                          /* tmatrices.h:307-309 */
    const qpms_tmatrix_interpolator_t *interp, double freq);
qpms_tmatrix_t *qpms_tmatrix_interpolator_eval(const qpms_tmatrix_interpolator_t *interp, double freq);
int qpms_tmatrix_generator_interpolator(qpms_tmatrix_t *t, qpms_complex_t omega,         /* tmatrices.h:326-330 */
    const void *interpolator);
const qpms_vswf_set_spec_t *qpms_tmatrix_interpolator_bspec(const qpms_tmatrix_interpolator_t *interp);
/* All elements of T(freqs[w]) for nf frequencies, out[w][n][n] row-major;
 * DEVICE pointers, stream-ordered on `stream` (a cudaStream_t). */
int qpms_gpu_tmatrix_interpolator_eval_batch(const qpms_tmatrix_interpolator_t *interp, size_t nf,
    const double *d_freqs, qpms_complex_t *d_out, void *stream);
/* SCUFF-EM T-matrix file (tmatrices.h:258-283, tmatrices.c:367-490): T-matrices
 * in the basis bs, frequencies in rad/s (and in SCUFF units); the arrays are
 * malloc'ed for the caller.  Returns QPMS_NAN_ENCOUNTERED if an element of the
 * basis is missing for some frequency. */
int qpms_load_scuff_tmatrix(const char *path, const qpms_vswf_set_spec_t *bs, size_t *n, double **freqs,
    double **freqs_su, qpms_tmatrix_t **tmatrices_array, qpms_complex_t **tmdata);

/* ---- T-matrices of axially symmetric particles (tmatrices.h:415-523) ----
 * Extended-boundary-condition method on the GPU: one CTA per (frequency, m)
 * integrates the Q and R blocks over composite Gauss-Legendre panels (broken
 * at the cylinder rims) and solves T = -R Q^-1 per m block; lMax_extend
 * (the internal basis, >= bspec lMax) up to 12.  The reference integrates each
 * entry by adaptive quadrature and warns that its results lose accuracy above
 * l = 1 (tmatrices.h:455-460); these reproduce the Mie T-matrix of a sphere to
 * double precision at every l. */
typedef struct qpms_arc_function_retval_t {                          /* tmatrices.h:415-419 */
  double r;     /* distance from the origin */
  double beta;  /* angle between the surface normal and the radial direction */
} qpms_arc_function_retval_t;
typedef struct qpms_arc_function_t {                                 /* tmatrices.h:421-435 */
  qpms_arc_function_retval_t (*function)(double theta, const void *params);
  const void *params;
} qpms_arc_function_t;
typedef struct qpms_arc_cylinder_params_t { double R, h; } qpms_arc_cylinder_params_t;  /* tmatrices.h:437-441 */
/* Spheroid with equatorial semi-axis a and polar (z) semi-axis c (no
 * counterpart in the reference, which takes it as a user arc function). */
typedef struct qpms_arc_spheroid_params_t { double a, c; } qpms_arc_spheroid_params_t;
qpms_arc_function_retval_t qpms_arc_cylinder(double theta, const void *params);  /* tmatrices.h:443-446 */
qpms_arc_function_retval_t qpms_arc_sphere(double theta, const void *R);          /* tmatrices.h:448-452 */
qpms_arc_function_retval_t qpms_arc_spheroid(double theta, const void *params);
/* Bridge for foreign-function callers that cannot return a struct from a
 * callback (ctypes): params -> {fn, user}, fn(theta, &r, &beta, user).  The
 * reference's Python layer wraps user arcs in Cython instead
 * (cytmatrices.pyx:164-168). */
typedef struct qpms_arc_callback_params_t {
  void (*fn)(double theta, double *r, double *beta, void *user);
  void *user;
} qpms_arc_callback_params_t;
qpms_arc_function_retval_t qpms_arc_callback(double theta, const void *params);
typedef struct qpms_tmatrix_generator_axialsym_param_t {             /* tmatrices.h:493-499 */
  qpms_epsmu_generator_t outside;
  qpms_epsmu_generator_t inside;
  qpms_arc_function_t shape;
  qpms_l_t lMax_extend;
} qpms_tmatrix_generator_axialsym_param_t;
/* Replace qpms_tmatrix_axialsym_fill / qpms_tmatrix_axialsym
 * (tmatrices.h:461-491, tmatrices.c:807-894). */
int qpms_tmatrix_axialsym_fill(qpms_tmatrix_t *t, qpms_complex_t omega, qpms_epsmu_t outside,
    qpms_epsmu_t inside, qpms_arc_function_t shape, qpms_l_t lMax_extend);
qpms_tmatrix_t *qpms_tmatrix_axialsym(const qpms_vswf_set_spec_t *bspec, qpms_complex_t omega,
    qpms_epsmu_t outside, qpms_epsmu_t inside, qpms_arc_function_t shape, qpms_l_t lMax_extend);
/* Replaces qpms_tmatrix_generator_axialsym (tmatrices.h:502-506, tmatrices.c:970-976). */
int qpms_tmatrix_generator_axialsym(qpms_tmatrix_t *t, qpms_complex_t omega, const void *params);
/* Replace the Q / R debugging fills (tmatrices.h:509-521, tmatrices.c:896-968):
 * target[i1 + i2 n] (n = 2 lMaxQR (lMaxQR + 2)) of the lMaxQR basis in
 * normalisation norm, J = QPMS_HANKEL_PLUS for Q, QPMS_BESSEL_REGULAR for R. */
int qpms_tmatrix_axialsym_RQ_transposed_fill(qpms_complex_t *target, qpms_complex_t omega,
    qpms_epsmu_t outside, qpms_epsmu_t inside, qpms_arc_function_t shape, qpms_l_t lMaxQR,
    qpms_normalisation_t norm, qpms_bessel_t J);
int qpms_tmatrix_generator_axialsym_RQ_transposed_fill(qpms_complex_t *target, qpms_complex_t omega,
    const qpms_tmatrix_generator_axialsym_param_t *param, qpms_normalisation_t norm, qpms_bessel_t J);
/* Batch (no counterpart): T of one shape at nw frequencies, outside[w] /
 * inside[w] the media there, into HOST T_out [nw][bspec->n][bspec->n]. */
int qpms_gpu_tmatrix_axialsym_batch(const qpms_vswf_set_spec_t *bspec, qpms_l_t lMax_extend,
    qpms_arc_function_t shape, size_t nw, const qpms_complex_t *omega, const qpms_epsmu_t *outside,
    const qpms_epsmu_t *inside, qpms_complex_t *T_out);

/* One particle kind of qpms_gpu_scatsys_create. */
typedef struct qpms_gpu_particle_kind_t {
  int type;             /* 0: sphere (Mie T-matrix), 1: tabulated T-matrix,
                           2: axially symmetric particle (T-matrix from its surface, GPU) */
  double radius;        /* sphere radius */
  qpms_complex_t eps;   /* types 0, 2: constant permittivity, used when neither ld nor eps_interp is set */
  const qpms_ldparams_t *ld;                             /* types 0, 2: Lorentz-Drude medium (copied) */
  const qpms_permittivity_interpolator_t *eps_interp;    /* types 0, 2: tabulated n, k (kept by reference) */
  const qpms_tmatrix_interpolator_t *tmatrix;            /* type 1: T(omega) in the lMax basis of the system
                                                             (kept by reference) */
  qpms_arc_function_t shape;   /* type 2: the surface (sampled once, at creation) */
  qpms_l_t lMax_extend;        /* type 2: internal basis of the Q, R matrices (>= lMax, <= 12) */
} qpms_gpu_particle_kind_t;

/* General constructor: np particles at pos_xyz, kind[i] in [0, nkinds),
 * constant medium, lMax basis (vswf.c:76-92); b1 = b2 = NULL for a finite
 * system, else a 2D lattice.  With tabulated T-matrix or axially symmetric
 * kinds every T is dense (spheres included); an axially symmetric kind's T
 * is formed on the GPU at every frequency the system is evaluated at.  Interpolated quantities
 * use Re omega (materials.c:131-142, tmatrices.c:351-356). */
qpms_scatsys_t *qpms_gpu_scatsys_create(int np, const double *pos_xyz, const int *kind, int nkinds,
    const qpms_gpu_particle_kind_t *kinds, qpms_complex_t eps_medium, qpms_l_t lMax,
    const double *b1, const double *b2);

/* Finite system of spheres with constant permittivities (Mie T-matrices,
 * tmatrices.c:580-606) in a constant medium; bspec from lMax (vswf.c:76-92).
 * kind[i] in [0, nkinds) selects radius[kind] and eps_inside[kind]. */
qpms_scatsys_t *qpms_gpu_scatsys_create_spheres(int np, const double *pos_xyz, const int *kind,
    int nkinds, const double *radius, const qpms_complex_t *eps_inside,
    qpms_complex_t eps_medium, qpms_l_t lMax);
void qpms_gpu_scatsys_free(qpms_scatsys_t *ss);

/* 2D-periodic system (lattice_dimension 2) with direct basis b1, b2 in the xy
 * plane; fills ss->per as process_lattice_bases does (scatsystem.c:187-214:
 * reduced basis, reciprocal basis, unit-cell area, eta = sqrt(pi / A)). */
qpms_scatsys_t *qpms_gpu_scatsys_create_spheres_2d(int np, const double *pos_xyz, const int *kind,
    int nkinds, const double *radius, const qpms_complex_t *eps_inside,
    qpms_complex_t eps_medium, qpms_l_t lMax, const double b1[2], const double b2[2]);

/* The same with dispersive spheres: kind t uses the Lorentz-Drude model
 * ld_inside[t] when that pointer is non-NULL (copied), else eps_inside[t]
 * (eps_inside may be NULL when every kind has a model); b1 = b2 = NULL for a
 * finite system, else a 2D lattice.  The T-matrices of every entry point
 * follow omega through the model. */
qpms_scatsys_t *qpms_gpu_scatsys_create_spheres_ld(int np, const double *pos_xyz, const int *kind, int nkinds,
    const double *radius, const qpms_complex_t *eps_inside, const qpms_ldparams_t *const *ld_inside,
    qpms_complex_t eps_medium, qpms_l_t lMax, const double *b1, const double *b2);

/* ---------------- point symmetry and irreps (scatsystem.h:300-430) ----------------
 * qpms_gpu_scatsys_set_symmetry gives a finite system one of the reference's
 * point groups generated by coordinate mirrors and rotations about z
 * ("trivial", "trivial_g", "C2", "C2v", "D2h", "x_and_z_flip",
 * "y_and_z_flip", "C4", "C4v", "D4h", "D3h"; symmetries.py point_group_info),
 * with its irrep names, irrep matrices and order (names sorted); the
 * two-dimensional E irreps pack to d x multiplicity vectors.  The packed (symmetry-adapted) basis is this
 * library's: packed vectors of the reference differ by a unitary change of
 * basis inside each irrep; eigenvalues, determinants and unpacked solutions
 * agree.  ss->saecv_sizes is set. */
int qpms_gpu_scatsys_set_symmetry(qpms_scatsys_t *ss, const char *group);
/* The same from the reference's group object (a qpms_finite_group_t *, whose
 * first member is the name, groups.h:53-54), e.g. the one
 * FinitePointGroup(point_group_info['D2h']) builds. */
int qpms_gpu_scatsys_set_symmetry_group(qpms_scatsys_t *ss, const void *finite_group);
int qpms_gpu_scatsys_nirreps(const qpms_scatsys_t *ss);
const char *qpms_gpu_scatsys_irrep_name(const qpms_scatsys_t *ss, int iri);
const size_t *qpms_gpu_scatsys_saecv_sizes(const qpms_scatsys_t *ss);
qpms_complex_t *qpms_scatsys_irrep_transform_matrix(qpms_complex_t *target_U,       /* scatsystem.h:313-314 */
    const qpms_scatsys_t *ss, int iri);
qpms_complex_t *qpms_scatsys_irrep_pack_matrix(qpms_complex_t *target_packed,       /* scatsystem.h:330-333 */
    const qpms_complex_t *orig_full, const qpms_scatsys_t *ss, int iri);
qpms_complex_t *qpms_scatsys_irrep_unpack_matrix(qpms_complex_t *target_full,       /* scatsystem.h:336-338 */
    const qpms_complex_t *orig_packed, const qpms_scatsys_t *ss, int iri, bool add);
qpms_complex_t *qpms_scatsys_irrep_pack_vector(qpms_complex_t *target_packed,       /* scatsystem.h:342-345 */
    const qpms_complex_t *orig_full, const qpms_scatsys_t *ss, int iri);
qpms_complex_t *qpms_scatsys_irrep_unpack_vector(qpms_complex_t *target_full,       /* scatsystem.h:348-351 */
    const qpms_complex_t *orig_packed, const qpms_scatsys_t *ss, int iri, bool add);
qpms_complex_t *qpms_scatsys_build_translation_matrix_e_irrep_packed(               /* scatsystem.h:390-397 */
    qpms_complex_t *target, const qpms_scatsys_t *ss, int iri, qpms_complex_t k, qpms_bessel_t J);
/* The reference's slow-implementation names and builder variants compute the
 * same (scatsystem.h:318-326, 413-430). */
qpms_complex_t *qpms_scatsys_irrep_pack_matrix_stupid(qpms_complex_t *target_packed,
    const qpms_complex_t *orig_full, const qpms_scatsys_t *ss, int iri);
qpms_complex_t *qpms_scatsys_irrep_unpack_matrix_stupid(qpms_complex_t *target_full,
    const qpms_complex_t *orig_packed, const qpms_scatsys_t *ss, int iri, bool add);
qpms_complex_t *qpms_scatsysw_build_modeproblem_matrix_irrep_packed_orbitorderR(qpms_complex_t *target,
    const qpms_scatsys_at_omega_t *ssw, int iri);
qpms_complex_t *qpms_scatsysw_build_modeproblem_matrix_irrep_packed_serial(qpms_complex_t *target,
    const qpms_scatsys_at_omega_t *ssw, int iri);

/* Evaluates the medium and the T-matrices at omega, like qpms_scatsys_at_omega
 * (scatsystem.c:606-630). */
qpms_scatsys_at_omega_t *qpms_gpu_scatsys_at_omega(const qpms_scatsys_t *ss, qpms_complex_t omega);
void qpms_gpu_scatsys_at_omega_free(qpms_scatsys_at_omega_t *ssw);
/* The reference's names of the lifetime functions (scatsystem.h:297-306):
 * qpms_scatsys_free, qpms_scatsys_at_omega, qpms_scatsys_at_omega_free. */
void qpms_scatsys_free(qpms_scatsys_t *ss);
qpms_scatsys_at_omega_t *qpms_scatsys_at_omega(const qpms_scatsys_t *ss, qpms_complex_t omega);
void qpms_scatsys_at_omega_free(qpms_scatsys_at_omega_t *ssw);
/* scatsystem.h:20: thread count of the reference's CPU builders; accepted and ignored. */
void qpms_scatsystem_set_nthreads(long n);

/* -- drop-in replacements of the reference's hot-path functions -- */

/* Irrep-packed mode problem (scatsystem.h:403-407, 451-473): assembled and
 * packed on the GPU; the LU and solve take packed vectors (qpms_ss_LU.full
 * false, .iri set). */
qpms_complex_t *qpms_scatsysw_build_modeproblem_matrix_irrep_packed(qpms_complex_t *target,
    const qpms_scatsys_at_omega_t *ssw, int iri);


/* Replaces qpms_scatsysw_build_modeproblem_matrix_full (scatsystem.h:368-372,
 * scatsystem.c:1345-1350): M = I - T S on the GPU (finite systems: S(R<-R) = 0,
 * the intended semantics of scatsystem.c:1283-1343).  target: host buffer of
 * fecv_size^2 (NULL -> malloc, caller frees). Returns target, NULL on error. */
qpms_complex_t *qpms_scatsysw_build_modeproblem_matrix_full(qpms_complex_t *target,
    const qpms_scatsys_at_omega_t *ssw);

/* Replaces qpms_scatsys_build_translation_matrix_e_full (scatsystem.h:357-363,
 * scatsystem.c:1180-1217): S(R<-C) of kind J for R != C, zero diagonal blocks. */
qpms_complex_t *qpms_scatsys_build_translation_matrix_e_full(qpms_complex_t *target,
    const qpms_scatsys_t *ss, qpms_complex_t k, qpms_bessel_t J);
/* Replaces qpms_scatsys_build_translation_matrix_full (scatsystem.h:357-362): J = QPMS_HANKEL_PLUS. */
qpms_complex_t *qpms_scatsys_build_translation_matrix_full(qpms_complex_t *target,
    const qpms_scatsys_t *ss, qpms_complex_t k);
/* Replace qpms_scatsys_periodic_build_translation_matrix_full and
 * qpms_scatsyswk_build_translation_matrix_full (scatsystem.h:505-519,
 * scatsystem.c:1252-1281): the lattice-summed W of the unit cell (2D xy
 * lattice); eta 0 / NaN selects qpms_ss_adjusted_eta. */
qpms_complex_t *qpms_scatsys_periodic_build_translation_matrix_full(qpms_complex_t *target,
    const qpms_scatsys_t *ss, qpms_complex_t wavenumber, const cart3_t *wavevector, double eta);
qpms_complex_t *qpms_scatsyswk_build_translation_matrix_full(qpms_complex_t *target,
    const qpms_scatsys_at_omega_k_t *sswk);

/* Replace qpms_scatsysw_modeproblem_matrix_full_factorise / _build_..._LU /
 * qpms_scatsys_scatter_solve / qpms_ss_LU_free (scatsystem.h:442-480,
 * scatsystem.c:2202-2273): LU with partial pivoting (zgetrf semantics,
 * row-major, 0-based ipiv) computed on the GPU; solve on the GPU. */
qpms_ss_LU qpms_scatsysw_modeproblem_matrix_full_factorise(qpms_complex_t *mpmatrix_full,
    int *target_piv, const qpms_scatsys_at_omega_t *ssw, const qpms_scatsys_at_omega_k_t *sswk);
qpms_ss_LU qpms_scatsysw_build_modeproblem_matrix_full_LU(qpms_complex_t *target,
    int *target_piv, const qpms_scatsys_at_omega_t *ssw);
qpms_ss_LU qpms_scatsysw_build_modeproblem_matrix_irrep_packed_LU(qpms_complex_t *target,
    int *target_piv, const qpms_scatsys_at_omega_t *ssw, int iri);
qpms_ss_LU qpms_scatsysw_modeproblem_matrix_irrep_packed_factorise(qpms_complex_t *mpmatrix_packed,
    int *target_piv, const qpms_scatsys_at_omega_t *ssw, int iri);
qpms_complex_t *qpms_scatsys_scatter_solve(qpms_complex_t *f, const qpms_complex_t *a_inc,
    qpms_ss_LU lu);
void qpms_ss_LU_free(qpms_ss_LU lu);

/* Replaces qpms_scatsysw_apply_Tmatrices_full (scatsystem.h:621-630,
 * scatsystem.c:1996-2011): target = T a per particle. */
qpms_complex_t *qpms_scatsysw_apply_Tmatrices_full(qpms_complex_t *target_full,
    const qpms_complex_t *inc_full, const qpms_scatsys_at_omega_t *ssw);

/* Replaces qpms_ss_adjusted_eta (scatsystem.h:795, scatsystem.c:68-80). */
double qpms_ss_adjusted_eta(const qpms_scatsys_t *ss, qpms_complex_t wavenumber, const double wavevector[3]);

/* Replaces qpms_scatsyswk_build_modeproblem_matrix_full (scatsystem.h:498-502,
 * scatsystem.c:1352-1357): M = I - T W(omega, k) of a 2D lattice, W from the
 * Ewald sums (short range, long range, sigma0) on the GPU; eta = sswk->eta or,
 * if 0/NaN, qpms_ss_adjusted_eta. */
qpms_complex_t *qpms_scatsyswk_build_modeproblem_matrix_full(qpms_complex_t *target,
    const qpms_scatsys_at_omega_k_t *sswk);
/* Replaces qpms_scatsyswk_build_modeproblem_matrix_full_LU (scatsystem.h:523-527). */
qpms_ss_LU qpms_scatsyswk_build_modeproblem_matrix_full_LU(qpms_complex_t *target, int *target_piv,
    const qpms_scatsys_at_omega_k_t *sswk);

/* Replace qpms_trans_calculator_get_AB_arrays_e32(_e) (translations.h:158-177,
 * translations.c:926-1078): lattice-summed A, B (2D xy lattice b1, b2, Bloch
 * vector beta, particle_shift, Ewald parameter eta) for the calculator's
 * normalisation, evaluated by the GPU Ewald kernel.  particle_shift.z != 0
 * (layers at different heights) takes the shifted-layer sums (the reference's
 * LAT_2D_IN_3D short-range branch and the shifted long-range branch,
 * ewald.c:441-469, marked untested there; here derived anew and checked by
 * eta invariance and direct summation).  parts must be
 * QPMS_EWALD_FULL (7).  maxR / maxK bound the lattice-point layers as in the
 * reference (PGen_xyWeb, latticegens.c:449-568): when those layers hold every
 * point whose term is above ~1e-16 of the leading one the result is the full
 * sum; a maxR / maxK that cuts into that region (a truncated sum) returns
 * QPMS_EINVAL with a message.  Aerr / Berr (optional) receive
 * |A(eta) - A(1.25 eta)| elementwise (B likewise): the eta-invariance of the
 * full sum as an estimate of its evaluation error. */
int qpms_trans_calculator_get_AB_arrays_e32(const qpms_trans_calculator *c,
    qpms_complex_t *Adest, double *Aerr, qpms_complex_t *Bdest, double *Berr,
    ptrdiff_t deststride, ptrdiff_t srcstride, double eta, qpms_complex_t wavenumber,
    cart2_t b1, cart2_t b2, cart2_t beta, cart3_t particle_shift, double maxR, double maxK);
int qpms_trans_calculator_get_AB_arrays_e32_e(const qpms_trans_calculator *c,
    qpms_complex_t *Adest, double *Aerr, qpms_complex_t *Bdest, double *Berr,
    ptrdiff_t deststride, ptrdiff_t srcstride, double eta, qpms_complex_t wavenumber,
    cart2_t b1, cart2_t b2, cart2_t beta, cart3_t particle_shift, double maxR, double maxK, int parts);

/* Batched dispersion scan of a 2D lattice (config "2D-periodic dispersion
 * scan"): for every omega (nw, real) and in-plane Bloch vector (nk, kvecs
 * [nk][2]) assemble M = I - T W (adjusted eta), LU-factorise and write
 * logdet[w][k] = log|det M| (from the factors: complex128 in mode 0,
 * complex64 in mode 1, about 1e-6 absolute); solve for the excitation of a
 * plane wave with in-plane wavevector = Bloch vector and E along x projected
 * perpendicular to k (x-polarised at normal incidence), in mode 1 with FP64
 * iterative refinement to 1e-13: f_out[w][k][fecv] (may be NULL),
 * sigma_ext = -Re(a^H f)/k^2 per cell, resid = ||M f - T a|| / ||T a||,
 * iters = applications of the factors.  Synchronous. */
int qpms_gpu_periodic_scan(const qpms_scatsys_t *ss, size_t nw, const double *omegas, size_t nk,
    const double *kvecs, int mode, double *logdet, qpms_complex_t *f_out, double *sigma_ext,
    double *resid_out, int *iters_out);

/* Plane-wave incident vector (qpms_scatsys_incident_field_vector_full with
 * qpms_incfield_planewave, scatsystem.c:1970-1983, vswf.c:480-530), real k. */
int qpms_gpu_incident_planewave_full(qpms_complex_t *target_full, const qpms_scatsys_t *ss,
    const double k_cart[3], const qpms_complex_t E_cart[3]);

/* Batched plane-wave scattering over frequencies (the loop of
 * misc/finiterectlat-scatter.py:70-111 on the full system): for each omega,
 * assemble M = I - T S, a = plane wave, solve M f = T a, sigma_ext =
 * -Re(a^H f)/k^2.  mode 0: plain FP64 (LU in complex128);  mode 1: LU in
 * complex64 with FP64 iterative refinement to the FP64 residual.
 * f_out (nw x fecv, host) may be NULL; resid_out[i] = ||M f - T a|| / ||T a||
 * (FP64); iters_out[i] = refinement steps (0 in mode 0).  Synchronous. */
int qpms_gpu_finite_planewave_scatter(const qpms_scatsys_t *ss, size_t nw,
    const double *omegas, const double k_dir[3], const qpms_complex_t E_cart[3], int mode,
    qpms_complex_t *f_out, double *sigma_ext, double *resid_out, int *iters_out);
/* The same with sigma_scat (may be NULL) = Re(f^H (I + R) f) / k^2, R the
 * regular-wave translation matrix with zero self blocks, the reference
 * script's scattering cross-section (misc/finiterectlat-scatter.py:98-111);
 * sigma_abs = sigma_ext - sigma_scat. */
int qpms_gpu_finite_planewave_scatter_ext(const qpms_scatsys_t *ss, size_t nw,
    const double *omegas, const double k_dir[3], const qpms_complex_t E_cart[3], int mode,
    qpms_complex_t *f_out, double *sigma_ext, double *sigma_scat, double *resid_out, int *iters_out);

/* ---------------- scattered field (scatsystem.h:700-790) ----------------
 * E(where) = sum over particles of the outgoing (btyp 3: Hankel h+) or other
 * (1 j, 2 y, 4 h-) VSWF expansion with the full coefficient vector cvf,
 * cartesian components.  Finite systems, default normalisation.  At a
 * particle centre the Hankel field is singular (non-finite), as in the
 * reference.  A failure returns a NaN field; qpms_gpu_last_error() tells why. */
ccart3_t qpms_scatsys_scattered_E(const qpms_scatsys_t *ss, qpms_bessel_t btyp,     /* scatsystem.c:2013-2039 */
    qpms_complex_t wavenumber, const qpms_complex_t *cvf, cart3_t where);
ccart3_t qpms_scatsysw_scattered_E(const qpms_scatsys_at_omega_t *ssw,            /* scatsystem.c:2041-2046 */
    qpms_bessel_t btyp, const qpms_complex_t *cvf, cart3_t where);
/* The reference's alternative route through the translation operator
 * (scatsystem.c:2048-2112) evaluates the same field; these run the direct kernel. */
ccart3_t qpms_scatsys_scattered_E__alt(const qpms_scatsys_t *ss, qpms_bessel_t btyp,
    qpms_complex_t wavenumber, const qpms_complex_t *cvf, cart3_t where);
ccart3_t qpms_scatsysw_scattered_E__alt(const qpms_scatsys_at_omega_t *ssw,
    qpms_bessel_t btyp, const qpms_complex_t *cvf, cart3_t where);
/* 2D-periodic system (scatsystem.c:2114-2188): the field of the lattice of
 * particles with Bloch vector sswk->k at any points (off the particles'
 * plane through the shifted-layer lattice sums), btyp 3 only (as in the
 * reference); sswk->eta = 0 selects qpms_ss_adjusted_eta. */
ccart3_t qpms_scatsyswk_scattered_E(const qpms_scatsys_at_omega_k_t *sswk, qpms_bessel_t btyp,
    const qpms_complex_t *cvf, cart3_t where);
int qpms_gpu_scatsyswk_scattered_E(const qpms_scatsys_at_omega_k_t *sswk, qpms_bessel_t btyp,
    const qpms_complex_t *cvf, size_t npoints, const double *where_xyz, qpms_complex_t *E_xyz);
/* Batched over points, HOST buffers (the loop of qpms_c.pyx:904-927 in one
 * call): where_xyz [npoints][3], E_xyz [npoints][3] complex. */
int qpms_gpu_scatsys_scattered_E(const qpms_scatsys_t *ss, qpms_bessel_t btyp,
    qpms_complex_t wavenumber, const qpms_complex_t *cvf, size_t npoints,
    const double *where_xyz, qpms_complex_t *E_xyz);
/* The same on DEVICE buffers, stream-ordered on `stream` (a cudaStream_t). */
int qpms_gpu_scatsys_scattered_E_device(const qpms_scatsys_t *ss, qpms_bessel_t btyp,
    qpms_complex_t wavenumber, const qpms_complex_t *d_cvf, size_t npoints,
    const double *d_where_xyz, qpms_complex_t *d_E_xyz, void *stream);

/* FP64-accurate residual R = B - M X (DEVICE pointers, complex128; M N x N
 * with leading dimension ldm, column-major or row-major; X, B, R N x nrhs
 * column-major) formed from bf16 digit products on the tensor cores, the
 * residual of the dense solver for nrhs >= 8.  No counterpart in the
 * reference (it calls zgetrs in FP64, scatsystem.c:2262-2273). */
int qpms_gpu_ozaki_residual(int N, int nrhs, const qpms_complex_t *M, size_t ldm, int row_major,
    const qpms_complex_t *X, const qpms_complex_t *B, qpms_complex_t *R);
/* C = A B for bf16 A (m x k), B (k x n) column-major and FP32 C on DEVICE
 * pointers: the cuBLAS call of the digit products, exposed for its exactness
 * test. */
int qpms_gpu_bf16_gemm(int m, int n, int k, const void *A, const void *B, float *C);

/* Dense complex solve X = M^-1 B on DEVICE pointers (column-major, any N):
 * random butterfly transform + blocked LU without pivoting;
 * mode 0 complex128 factors (plain FP64), mode 1 complex64 factors
 * (tensor-core GEMMs); both refined with FP64 residuals to 1e-13.  The solver
 * of the Beyn contour nodes (the reference factorises with
 * LAPACKE_zgetrf/zgetrs, beyn.c:552-564).  resid = ||B - M X||_F / ||B||_F
 * (FP64), iters = applications of the factors.  Synchronous. */
int qpms_gpu_dense_solve(int N, int nrhs, const qpms_complex_t *M, const qpms_complex_t *B,
    qpms_complex_t *X, int mode, double *resid, int *iters);

/* Complex64 GEMM on the tensor cores (tcgen05, TMA-staged operands):
 * D = beta C + alpha A B with A (m x k), B (k x n), C, D (m x n) complex64
 * (interleaved float pairs), column-major, leading dimensions in complex
 * elements, device pointers, asynchronous on `stream` (C == D allowed; C is
 * not read when beta == 0).  Operands are cut into nsplit bf16 digits
 * (1, 2 or 3) and the digit products with s + t < nsplit are accumulated in
 * FP32: relative error about 4e-3, 2e-5 and 2e-7.  The building block of the
 * mixed-precision LU that replaces the reference's LAPACKE_zgetrf / zgetrs
 * (scatsystem.c:2202-2273, beyn.c:552-564).  Allocates its digit planes with
 * cudaMallocAsync on the stream. */
int qpms_gpu_tc_cgemm(int m, int n, int k, const void *A, size_t lda, const void *B, size_t ldb,
    float alpha, float beta, const void *C, size_t ldc, void *D, size_t ldd, int nsplit, void *stream);

/* Real bf16 GEMM on the tensor cores with FP32 output: D = beta C + alpha A B^T,
 * A [m][k] and B [n][k] row-major bf16 (row strides lda, ldb: multiples of 8),
 * D (and C) m x n column-major float.  The digit products of the FP64
 * refinement residual use it (exact for integer operands whose products sum
 * below 2^24). */
int qpms_gpu_tc_gemm_bf16(int m, int n, int k, const void *A, size_t lda, const void *B, size_t ldb,
    float alpha, float beta, const float *C, size_t ldc, float *D, size_t ldd, void *stream);

/* Live kernel timing for measurements (off by default): enable != 0 starts
 * recording a CUDA event pair around every launch of the library's main
 * kernels, on the stream each is launched on, with the launch's work; 0 stops.
 * Either call clears the sums.  Kinds: 0 tensor-core GEMM (work: executed
 * bf16 flops), 1 finite assembly (matrix bytes), 2 lattice-sum assembly
 * (matrix bytes), 3 batched small LU (complex flops 8 N^3 / 3), 4 dense
 * diagonal-block LU (8 nb^3 / 3), 5 translation coefficients (output bytes),
 * 6 digit splitting (bytes written).  _get synchronises the recorded events
 * and returns the summed device milliseconds, work and launch count. */
int qpms_gpu_kernel_timing(int enable);
int qpms_gpu_kernel_timing_get(int kind, double *ms, double *work, unsigned long long *launches);

/* QPMS_ERROR (with a message) if a tensor-core kernel's pipeline wait ran out
 * of time since the last check; synchronises the stream and clears the flag. */
int qpms_gpu_tc_check_error(void *stream);

/* ---------------- Beyn contour-integral eigensolver (beyn.h) ---------------- */
#define QPMS_NO_IRREP ((qpms_iri_t) -1)   /* qpms_types.h:325 */

/* M(z) into target (row-major m x m), beyn.h:22. */
typedef int (*beyn_function_M_t)(qpms_complex_t *target_M, size_t m, qpms_complex_t z, void *params);
/* M(z)^-1 Vhat (row-major m x l), beyn.h:26-27. */
typedef int (*beyn_function_M_inv_Vhat_t)(qpms_complex_t *target_M_inv_Vhat, size_t m, size_t l,
    const qpms_complex_t *Vhat, qpms_complex_t z, void *params);

/* Integration contour, beyn.h:30-43: n nodes (z, dz) followed by one hidden
 * entry holding the half-axes of an ellipse. */
typedef struct beyn_contour_t {
  size_t n;
  qpms_complex_t centre;
  bool (*inside_test)(struct beyn_contour_t *, qpms_complex_t z);
  qpms_complex_t z_dz[][2];
} beyn_contour_t;

/* beyn.h:47 (beyn.c:69-86); free with free(). */
beyn_contour_t *beyn_contour_ellipse(qpms_complex_t centre, double halfax_re, double halfax_im, size_t npoints);

/* Result, beyn.h:82-94: neig eigenvalues, their error estimates (coarse minus
 * fine contour), residuals |M(z) v|, eigenvectors as rows of length vlen, and
 * the singular values of the rank test.  `gsl` is private here (NULL). */
typedef struct beyn_result_t {
  size_t neig;
  size_t vlen;
  qpms_complex_t *eigval;
  qpms_complex_t *eigval_err;
  double *residuals;
  qpms_complex_t *eigvec;
  double *ranktest_SV;
  void *gsl;
} beyn_result_t;

/* beyn.h:101 */
void beyn_result_free(beyn_result_t *result);

/* beyn.h:115-125 (beyn.c:625-634 over beyn_solve_gsl, beyn.c:471-584).  The
 * quadrature solves M(z_i) X = Vhat on the GPU (one LU per node, L right-hand
 * sides, complex64 factors with FP64 iterative refinement); M comes from the
 * host callback.  The probe matrix Vhat is drawn from a fixed seed (the
 * reference seeds from the clock, beyn.c:292).  M_inv_Vhat, when given, is
 * used in place of the LU as in the reference. */
beyn_result_t *beyn_solve(size_t m, size_t l, beyn_function_M_t M, beyn_function_M_inv_Vhat_t M_inv_Vhat,
    void *params, const beyn_contour_t *contour, double rank_tol, size_t rank_sel_min, double res_tol);

/* scatsystem.h:649-662 (scatsystem.c:2301-2324): eigenmodes of a finite
 * system inside an ellipse in the complex omega plane, l = fecv_size probe
 * columns as in the reference; iri = QPMS_NO_IRREP for the full M, else M
 * projected on that irrep of the system's point group (saecv_sizes[iri]
 * probe columns, eigenvectors in the packed basis).  M(omega) is assembled
 * (and packed) on the GPU. */
beyn_result_t *qpms_scatsys_finite_find_eigenmodes(const qpms_scatsys_t *ss, qpms_iri_t iri,
    qpms_complex_t omega_centre, double omega_rr, double omega_ri, size_t contour_npoints,
    double rank_tol, size_t rank_sel_min, double res_tol);

/* scatsystem.h:538-549 (scatsystem.c:2351-2372): the same for a 2D-periodic
 * system at Bloch vector k, M = I - T W(omega, k) with the adjusted Ewald eta. */
beyn_result_t *qpms_scatsys_periodic_find_eigenmodes(const qpms_scatsys_t *ss, const double k[3],
    qpms_complex_t omega_centre, double omega_rr, double omega_ri, size_t contour_npoints,
    double rank_tol, size_t rank_sel_min, double res_tol);

/* Extended form of the two above (k = NULL: finite system): l probe columns
 * (l <= fecv_size), Vhat (row-major fecv_size x l, or NULL for the seeded
 * generator), mode 0 = plain FP64 LU per node, 1 = complex64 LU with FP64
 * refinement to refine_tol (relative residual; <= 0 selects 1e-12).
 * rank_tol < 0 selects a relative rank test (extended entry points only):
 * singular values above |rank_tol| * sum_i |dz_i| * ||Vhat||_F / sqrt(l), the
 * size of the quadrature sums without cancellation -- with no eigenvalue
 * inside the contour they are cancellation noise near 1e-16 of it, which the
 * reference's absolute threshold cannot tell from a mode when omega ~ 1e15.
 * The drop-ins above keep the absolute test (negative values act as 0). */
beyn_result_t *qpms_gpu_scatsys_find_eigenmodes(const qpms_scatsys_t *ss, const double *k,
    qpms_complex_t omega_centre, double omega_rr, double omega_ri, size_t contour_npoints,
    double rank_tol, size_t rank_sel_min, double res_tol, size_t l, const qpms_complex_t *Vhat,
    unsigned long long seed, int mode, double refine_tol);

/* The extended form on irrep iri of a finite system with point symmetry
 * (l <= saecv_sizes[iri], Vhat saecv_sizes[iri] x l). */
beyn_result_t *qpms_gpu_scatsys_find_eigenmodes_irrep(const qpms_scatsys_t *ss, int iri,
    qpms_complex_t omega_centre, double omega_rr, double omega_ri, size_t contour_npoints,
    double rank_tol, size_t rank_sel_min, double res_tol, size_t l, const qpms_complex_t *Vhat,
    unsigned long long seed, int mode, double refine_tol);

/* Extended beyn_solve: explicit probe matrix / seed and precision mode. */
beyn_result_t *qpms_gpu_beyn_solve(size_t m, size_t l, beyn_function_M_t M, void *params,
    const beyn_contour_t *contour, double rank_tol, size_t rank_sel_min, double res_tol,
    const qpms_complex_t *Vhat, unsigned long long seed, int mode, double refine_tol);

/* Sharding the contour over processes or devices (replicas with one exchange
 * step): each part sums nodes [node_begin, node_end) of the contour into the
 * host column-major fecv_size x l arrays A0, A1 and the coarse A0c, A1c (the
 * parts add up to the full quadrature; Vhat / seed as above, identical on
 * every part); the summed arrays then go to qpms_gpu_beyn_process (host only,
 * no residual filter) on one process.  No counterpart in the reference. */
int qpms_gpu_scatsys_beyn_quadrature(const qpms_scatsys_t *ss, const double *k, const beyn_contour_t *contour,
    size_t node_begin, size_t node_end, size_t l, const qpms_complex_t *Vhat, unsigned long long seed, int mode,
    double refine_tol, qpms_complex_t *A0, qpms_complex_t *A1, qpms_complex_t *A0c, qpms_complex_t *A1c);
beyn_result_t *qpms_gpu_beyn_process(size_t m, size_t l, const qpms_complex_t *A0, const qpms_complex_t *A1,
    const qpms_complex_t *A0c, const qpms_complex_t *A1c, qpms_complex_t z0, double rank_tol,
    size_t rank_sel_min);

/* Diagnostics of a result made here: largest FP64 relative residual of the
 * node solves, most refinement steps of one node, wall time of the contour
 * quadrature and of the whole solve (seconds). */
int qpms_gpu_beyn_result_stats(const beyn_result_t *result, double *max_node_resid, int *max_node_iters,
    double *quadrature_s, double *total_s);

/* The seeded probe matrix (row-major m x l, complex Gaussian) used when no
 * Vhat is given, so that callers can reproduce it. */
int qpms_gpu_beyn_probe_matrix(size_t m, size_t l, unsigned long long seed, qpms_complex_t *out);

/* Host linear algebra of the Beyn post-processing, exposed for tests:
 * thin SVD (column-major m x n, m >= n) and general eigenproblem (n x n). */
int qpms_gpu_host_svd(int m, int n, const qpms_complex_t *A, qpms_complex_t *U, double *s, qpms_complex_t *V);
int qpms_gpu_host_eig(int n, const qpms_complex_t *A, qpms_complex_t *w, qpms_complex_t *X);

/* ---------------- serving loop (continuous batching) ---------------- */
/* One plane-wave scattering solve (the unit of work of the reference's
 * misc/finiterectlat-scatter.py and misc/infiniterectlat-scatter.py loops):
 * a finite system at omega with incidence direction k_dir and polarisation E,
 * or a 2D-periodic system at omega and in-plane Bloch vector k (incidence with
 * that in-plane wavevector, x polarisation projected perpendicular to it).
 * Systems come from qpms_gpu_scatsys_create_spheres[_2d].  No counterpart in
 * the reference, which solves one request at a time. */
typedef struct qpms_gpu_request_t {
  const qpms_scatsys_t *ss;
  double omega;
  double k[2];
  double k_dir[3];
  qpms_complex_t E[3];
} qpms_gpu_request_t;

typedef struct qpms_gpu_result_t {
  int status;                    /* 0 = solved; QPMS_ECANCELED if cancelled before it started */
  int iters;                     /* refinement steps (mixed mode) */
  int batch_size;                /* requests solved together with this one */
  int fallback;                  /* 1: the mixed-precision refinement stalled and the system was solved
                                    again with more precise factors (complex128 at the end) */
  double sigma_ext;              /* extinction cross-section (per unit cell if periodic) */
  double residual;               /* FP64 relative residual |b - M x| / |b| */
  double t_submit, t_start, t_done;   /* seconds on the server clock */
} qpms_gpu_result_t;

typedef struct qpms_gpu_server qpms_gpu_server_t;

/* A serving loop on the current device: `workers` threads with one stream
 * each, device memory from a private pool, requests admitted while their
 * footprint fits hbm_budget_bytes (0: 60 % of free memory).  mode 1 solves in
 * complex64 with FP64 refinement, mode 0 in plain complex128. */
qpms_gpu_server_t *qpms_gpu_server_create(size_t hbm_budget_bytes, int mode, int workers);
/* Queue a request; f_out (fecv_size complex, host, may be NULL) receives the
 * scattered-field coefficients and must stay valid until qpms_gpu_server_wait. */
int qpms_gpu_server_submit(qpms_gpu_server_t *s, const qpms_gpu_request_t *req, qpms_complex_t *f_out,
    uint64_t *ticket);
/* Block until the request is solved; returns its status. */
int qpms_gpu_server_wait(qpms_gpu_server_t *s, uint64_t ticket, qpms_gpu_result_t *out);
/* Withdraw a request that has not started: it completes with status
 * QPMS_ECANCELED (its ticket must still be waited for).  Returns 0, or
 * QPMS_EINVAL if the ticket is unknown or the request has already started. */
int qpms_gpu_server_cancel(qpms_gpu_server_t *s, uint64_t ticket);
/* Block until nothing is queued or running. */
int qpms_gpu_server_drain(qpms_gpu_server_t *s);
/* Test hook: the next `count` device-pool allocations of the server's
 * workers fail as if the pool were exhausted (the affected request completes
 * with QPMS_ENOMEM; the server keeps serving).  No counterpart in the reference. */
int qpms_gpu_server_testing_fail_allocations(qpms_gpu_server_t *s, int count);
/* Test hook: caps the FP64 refinement steps of the mixed-precision solves
 * (batched and dense) at max_steps (-1 restores the default), so that tests
 * can force the precision fallback.  No counterpart in the reference. */
int qpms_gpu_testing_set_max_refine(int max_steps);
double qpms_gpu_server_clock(qpms_gpu_server_t *s);
int qpms_gpu_server_stats(qpms_gpu_server_t *s, size_t *completed, size_t *batches, size_t *peak_bytes,
    int *max_concurrent, size_t *budget_bytes);
/* Stops the workers (drain first: queued requests are dropped). */
void qpms_gpu_server_destroy(qpms_gpu_server_t *s);

/* ---------------- diagnostics ---------------- */
/* Thread-local message of the last failing call (empty string if none). */
const char *qpms_gpu_last_error(void);
/* FP64 FMA throughput of the current device in TFLOP/s (probe kernel), the
 * denominator of FP64-pipe roofline fractions.  No counterpart in the reference. */
int qpms_gpu_measure_fp64_peak(double *tflops);
/* Host evaluation of the library's complex erfc (Weideman Faddeeva), for tests. */
int qpms_gpu_debug_cerfc(double re, double im, double *out);
/* Number of kernels this library launched since load (for benchmarks); the
 * launches inside a replayed CUDA graph count as well. */
unsigned long long qpms_gpu_kernel_launch_count(void);
/* Number of CUDA-graph replays since load: the dense solver of the Beyn node
 * loop captures its factorisation and solve launch sequences once and replays
 * them at the following nodes (QPMS_GB300_GRAPHS=0 turns this off). */
unsigned long long qpms_gpu_graph_replay_count(void);

/* ---------------- reference-API convenience entry points ----------------
 * Host set-up helpers beside the hot path (qg_dropins.cu): O(n) or O(n^2) per
 * particle or contour.  The reference defines several of them as static
 * inline functions (materials.h, tmatrices.h:380-412); exported here so that
 * foreign-function callers can bind them. */
typedef struct sph_t { double r, theta, phi; } sph_t;                        /* qpms_types.h:207-209 */
typedef struct csphvec_t { qpms_complex_t rc, thetac, phic; } csphvec_t;     /* qpms_types.h:218-220 */

/* materials.h:40-55, 28-34, 151-158; materials.c:166-177 */
qpms_complex_t qpms_refindex(qpms_epsmu_t em);
qpms_complex_t qpms_wavenumber(qpms_complex_t omega, qpms_epsmu_t em);
qpms_complex_t qpms_waveimpedance(qpms_epsmu_t em);
qpms_epsmu_t qpms_epsmu_generator_eval(qpms_epsmu_generator_t gen, qpms_complex_t omega);
qpms_complex_t qpms_drude_epsilon(qpms_complex_t eps_inf, qpms_complex_t omega_p, qpms_complex_t gamma_p,
    qpms_complex_t omega);
qpms_epsmu_t qpms_lorentzdrude_epsmu(qpms_complex_t omega, const qpms_ldparams_t *p);
qpms_epsmu_t qpms_lorentzdrude_epsmu_g(qpms_complex_t omega, const void *p);

/* Sphere T-matrices (tmatrices.h:345-412, tmatrices.c:500-606).  Bessel
 * orders are compiled up to lMax 10 here; a larger lMax, equal J_ext and
 * J_scat, or a longitudinal basis element returns NULL / QPMS_EINVAL with a
 * message (the reference aborts on the first two). */
qpms_complex_t *qpms_mie_coefficients_reflection(qpms_complex_t *target, const qpms_vswf_set_spec_t *bspec,
    double a, qpms_complex_t k_i, qpms_complex_t k_e, qpms_complex_t mu_i, qpms_complex_t mu_e,
    qpms_bessel_t J_ext, qpms_bessel_t J_scat);
int qpms_tmatrix_spherical_fill(qpms_tmatrix_t *t, double a, qpms_complex_t k_i, qpms_complex_t k_e,
    qpms_complex_t mu_i, qpms_complex_t mu_e);
qpms_tmatrix_t *qpms_tmatrix_spherical(const qpms_vswf_set_spec_t *bspec, double a, qpms_complex_t k_i,
    qpms_complex_t k_e, qpms_complex_t mu_i, qpms_complex_t mu_e);
int qpms_tmatrix_spherical_mu0_fill(qpms_tmatrix_t *t, double a, double omega, qpms_complex_t epsilon_fg,
    qpms_complex_t epsilon_bg);
qpms_tmatrix_t *qpms_tmatrix_spherical_mu0(const qpms_vswf_set_spec_t *bspec, double a, double omega,
    qpms_complex_t epsilon_fg, qpms_complex_t epsilon_bg);
typedef struct qpms_tmatrix_generator_sphere_param_t {               /* tmatrices.h:367-371 */
  qpms_epsmu_generator_t outside;
  qpms_epsmu_generator_t inside;
  double radius;
} qpms_tmatrix_generator_sphere_param_t;
int qpms_tmatrix_generator_sphere(qpms_tmatrix_t *t, qpms_complex_t omega, const void *params);  /* tmatrices.h:374-377 */
/* T-matrix generators and helpers (tmatrices.h:22-45, 245-281; tmatrices.c:49-75, 257-271, 608-619, 980-989) */
typedef struct qpms_tmatrix_generator_t {                            /* tmatrices.h:258-264 */
  int (*function)(qpms_tmatrix_t *t, qpms_complex_t omega, const void *params);
  const void *params;
} qpms_tmatrix_generator_t;
qpms_tmatrix_t *qpms_tmatrix_init_from_generator(const qpms_vswf_set_spec_t *bspec, qpms_tmatrix_generator_t gen,
    qpms_complex_t omega);
int qpms_tmatrix_generator_constant(qpms_tmatrix_t *t, qpms_complex_t omega, const void *tmatrix_orig);
qpms_tmatrix_t *qpms_tmatrix_copy(const qpms_tmatrix_t *T);
qpms_tmatrix_t *qpms_tmatrix_mv(qpms_tmatrix_t *dest, const qpms_tmatrix_t *orig);
bool qpms_tmatrix_isclose(const qpms_tmatrix_t *T1, const qpms_tmatrix_t *T2, double rtol, double atol);
qpms_complex_t *qpms_apply_tmatrix(qpms_complex_t *f_target, const qpms_complex_t *a, const qpms_tmatrix_t *T);

/* Plane waves (vswf.h:92-126, 229-234; vswf.c:445-530).  Longitudinal
 * coefficients are zero for a transverse amplitude (rc == 0); a
 * non-transverse amplitude with a longitudinal target returns QPMS_EINVAL.
 * qpms_incfield_planewave takes the direction of Re k and multiplies the
 * expansion by e^{i k . evalpoint} (complex k included). */
int qpms_planewave2vswf_fill_cart(cart3_t wavedir, ccart3_t amplitude, qpms_complex_t *target_longcoeff,
    qpms_complex_t *target_mgcoeff, qpms_complex_t *target_elcoeff, qpms_l_t lMax, qpms_normalisation_t norm);
int qpms_planewave2vswf_fill_sph(sph_t wavedir, csphvec_t amplitude, qpms_complex_t *target_longcoeff,
    qpms_complex_t *target_mgcoeff, qpms_complex_t *target_elcoeff, qpms_l_t lMax, qpms_normalisation_t norm);
typedef int (*qpms_incfield_t)(qpms_complex_t *target, const qpms_vswf_set_spec_t *bspec,  /* vswf.h:17-24 */
    const cart3_t evalpoint, const void *args, bool add);
typedef struct qpms_incfield_planewave_params_t {                    /* vswf.h:93-103 */
  bool use_cartesian;
  union { ccart3_t cart; csph_t sph; } k;
  union { ccart3_t cart; csphvec_t sph; } E;
} qpms_incfield_planewave_params_t;
int qpms_incfield_planewave(qpms_complex_t *target, const qpms_vswf_set_spec_t *bspec, const cart3_t evalpoint,
    const void *args, bool add);
/* scatsystem.h:621-629, scatsystem.c:1970-1983: field_at_point per particle
 * into its slice of the full vector (allocated with calloc when NULL). */
qpms_complex_t *qpms_scatsys_incident_field_vector_full(qpms_complex_t *target_full, const qpms_scatsys_t *ss,
    qpms_incfield_t field_at_point, const void *args, bool add);

/* Single translation coefficients (translations.h:40-44, 93-121): taken from
 * one GPU evaluation of the A / B arrays; A(m n <- mu nu) is the
 * [y(m, n)][y(mu, nu)] element of qpms_trans_calculator_get_AB_arrays.  An
 * out-of-range index returns QPMS_EINVAL (NaN for the value-returning forms). */
qpms_complex_t qpms_trans_single_A(qpms_normalisation_t norm, qpms_m_t m, qpms_l_t n, qpms_m_t mu, qpms_l_t nu,
    csph_t kdlj, bool r_ge_d, qpms_bessel_t J);
qpms_complex_t qpms_trans_single_B(qpms_normalisation_t norm, qpms_m_t m, qpms_l_t n, qpms_m_t mu, qpms_l_t nu,
    csph_t kdlj, bool r_ge_d, qpms_bessel_t J);
qpms_complex_t qpms_trans_calculator_get_A(const qpms_trans_calculator *c, qpms_m_t m, qpms_l_t n, qpms_m_t mu,
    qpms_l_t nu, csph_t kdlj, bool r_ge_d, qpms_bessel_t J);
qpms_complex_t qpms_trans_calculator_get_B(const qpms_trans_calculator *c, qpms_m_t m, qpms_l_t n, qpms_m_t mu,
    qpms_l_t nu, csph_t kdlj, bool r_ge_d, qpms_bessel_t J);
int qpms_trans_calculator_get_AB_p(const qpms_trans_calculator *c, qpms_complex_t *Adest, qpms_complex_t *Bdest,
    qpms_m_t m, qpms_l_t n, qpms_m_t mu, qpms_l_t nu, csph_t kdlj, bool r_ge_d, qpms_bessel_t J);
qpms_complex_t qpms_trans_calculator_get_A_ext(const qpms_trans_calculator *c, int m, int n, int mu, int nu,
    qpms_complex_t kdlj_r, double kdlj_th, double kdlj_phi, int r_ge_d, int J);
qpms_complex_t qpms_trans_calculator_get_B_ext(const qpms_trans_calculator *c, int m, int n, int mu, int nu,
    qpms_complex_t kdlj_r, double kdlj_th, double kdlj_phi, int r_ge_d, int J);
int qpms_trans_calculator_get_AB_p_ext(const qpms_trans_calculator *c, qpms_complex_t *Adest,
    qpms_complex_t *Bdest, int m, int n, int mu, int nu, qpms_complex_t kdlj_r, double kdlj_th,
    double kdlj_phi, int r_ge_d, int J);

/* Half-ellipse and kidney contours (beyn.h:50-66, beyn.c:117-226): n nodes,
 * the half-axes in entry n and the orientation after it; inside_test NULL. */
typedef int beyn_contour_halfellipse_orientation;                   /* beyn.h:50-55 */
#define BEYN_CONTOUR_HALFELLIPSE_RE_PLUS 3
#define BEYN_CONTOUR_HALFELLIPSE_RE_MINUS 1
#define BEYN_CONTOUR_HALFELLIPSE_IM_PLUS 0
#define BEYN_CONTOUR_HALFELLIPSE_IM_MINUS 2
beyn_contour_t *beyn_contour_halfellipse(qpms_complex_t centre, double halfax_re, double halfax_im,
    size_t npoints, beyn_contour_halfellipse_orientation orientation);
beyn_contour_t *beyn_contour_kidney(qpms_complex_t centre, double halfax_re, double halfax_im, double rounding,
    size_t n, beyn_contour_halfellipse_orientation orientation);

#ifdef __cplusplus
}
#endif
#endif
