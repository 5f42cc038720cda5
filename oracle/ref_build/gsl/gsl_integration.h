/* GSL stand-in (test infrastructure): QAGS / QAGIU with a workspace handle. */
#ifndef FJREF_GSL_INTEGRATION_H
#define FJREF_GSL_INTEGRATION_H
#include <stddef.h>
#include "gsl_math.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { size_t limit; } gsl_integration_workspace;
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
int gsl_integration_qags(const gsl_function *f, double a, double b, double epsabs, double epsrel,
                         size_t limit, gsl_integration_workspace *w, double *result, double *abserr);
int gsl_integration_qagiu(gsl_function *f, double a, double epsabs, double epsrel, size_t limit,
                          gsl_integration_workspace *w, double *result, double *abserr);
#ifdef __cplusplus
}
#endif
#endif
