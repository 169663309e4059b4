/* Test-only GSL error declarations for the oracle pin build. */
#ifndef GWO_SHIM_GSL_ERRNO_H
#define GWO_SHIM_GSL_ERRNO_H
#define GSL_SUCCESS 0
#define GSL_EDOM 1
#define GSL_EINVAL 4
#define GSL_EFAILED 5
#define GSL_ENOMEM 8
typedef void gsl_error_handler_t(const char *, const char *, int, int);
static inline gsl_error_handler_t *gsl_set_error_handler_off(void) { return 0; }
static inline const char *gsl_strerror(const int gsl_errno) { (void)gsl_errno; return "gsl error"; }
#endif
