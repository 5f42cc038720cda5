/* GSL stand-in (test infrastructure): the subset of <gsl/gsl_errno.h> the reference uses. */
#ifndef FJREF_GSL_ERRNO_H
#define FJREF_GSL_ERRNO_H
#ifdef __cplusplus
extern "C" {
#endif
#define GSL_SUCCESS 0
#define GSL_CONTINUE (-2)
typedef void gsl_error_handler_t(const char *reason, const char *file, int line, int gsl_errno);
gsl_error_handler_t *gsl_set_error_handler_off(void);
#ifdef __cplusplus
}
#endif
#endif
