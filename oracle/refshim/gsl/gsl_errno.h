/* Minimal stand-in for GSL's gsl_errno.h (oracle test infrastructure). */
#ifndef QG_REFSHIM_GSL_ERRNO_H
#define QG_REFSHIM_GSL_ERRNO_H
#include <errno.h>
#include <stdio.h>
enum { GSL_SUCCESS = 0, GSL_FAILURE = -1, GSL_EDOM = 1, GSL_ERANGE = 2, GSL_EINVAL = 4, GSL_EFAILED = 5,
       GSL_ENOMEM = 8, GSL_EMAXITER = 11, GSL_ETOL = 14, GSL_EUNDRFLW = 15, GSL_EOVRFLW = 16, GSL_EROUND = 18 };
#define GSL_ERROR(reason, gsl_errno)                  \
  do {                                                 \
    gsl_error(reason, __FILE__, __LINE__, gsl_errno); \
    return gsl_errno;                                  \
  } while (0)
#define GSL_ERROR_SELECT_2(a, b) ((a) != GSL_SUCCESS ? (a) : ((b) != GSL_SUCCESS ? (b) : GSL_SUCCESS))
typedef void gsl_error_handler_t(const char *reason, const char *file, int line, int gsl_errno);
gsl_error_handler_t *gsl_set_error_handler(gsl_error_handler_t *new_handler);
gsl_error_handler_t *gsl_set_error_handler_off(void);
void gsl_error(const char *reason, const char *file, int line, int gsl_errno);
void gsl_stream_printf(const char *label, const char *file, int line, const char *reason);
const char *gsl_strerror(const int gsl_errno);
#endif
