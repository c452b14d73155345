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
#define QPMS_NORMALISATION_CSPHASE 8
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

/* Number of A / B multipliers (ragged table sizes), for tests. */
size_t qpms_gpu_trans_calculator_n_multipliers(const qpms_trans_calculator *c, int which_B);

/* Host-only export of the ragged A/B multiplier tables of
 * qpms_trans_calculator_init (same order as the reference's
 * A_multipliers[0][...], translations.c:464-471), computed without a GPU.
 * *nA, *nB: capacity on input, table size on output; NULL outputs query sizes. */
int qpms_gpu_trans_multipliers_export(qpms_l_t lMax, qpms_normalisation_t nt,
    qpms_complex_t *A_out, size_t *nA, qpms_complex_t *B_out, size_t *nB);

/* ---------------- diagnostics ---------------- */
/* Thread-local message of the last failing call (empty string if none). */
const char *qpms_gpu_last_error(void);
/* FP64 FMA throughput of the current device in TFLOP/s (probe kernel), the
 * denominator of FP64-pipe roofline fractions.  No counterpart in the reference. */
int qpms_gpu_measure_fp64_peak(double *tflops);
/* Number of kernels this library launched since load (for benchmarks). */
unsigned long long qpms_gpu_kernel_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif
