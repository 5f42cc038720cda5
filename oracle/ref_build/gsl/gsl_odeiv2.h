/* GSL stand-in (test infrastructure): adaptive ODE evolution interface.  The
   "rk8pd" stepper is the RK8(7) pair of Prince & Dormand (see gsl_standin.c). */
#ifndef FJREF_GSL_ODEIV2_H
#define FJREF_GSL_ODEIV2_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct {
    int (*function)(double t, const double y[], double dydt[], void *params);
    int (*jacobian)(double t, const double y[], double *dfdy, double dfdt[], void *params);
    size_t dimension;
    void *params;
} gsl_odeiv2_system;
typedef struct fjref_step_type gsl_odeiv2_step_type;
typedef struct fjref_step gsl_odeiv2_step;
typedef struct fjref_control gsl_odeiv2_control;
typedef struct fjref_evolve gsl_odeiv2_evolve;
extern const gsl_odeiv2_step_type *gsl_odeiv2_step_rk8pd;
gsl_odeiv2_step *gsl_odeiv2_step_alloc(const gsl_odeiv2_step_type *T, size_t dim);
gsl_odeiv2_control *gsl_odeiv2_control_y_new(double eps_abs, double eps_rel);
gsl_odeiv2_evolve *gsl_odeiv2_evolve_alloc(size_t dim);
int gsl_odeiv2_evolve_apply(gsl_odeiv2_evolve *e, gsl_odeiv2_control *con, gsl_odeiv2_step *step,
                            const gsl_odeiv2_system *sys, double *t, double t1, double *h, double y[]);
void gsl_odeiv2_evolve_free(gsl_odeiv2_evolve *e);
void gsl_odeiv2_control_free(gsl_odeiv2_control *c);
void gsl_odeiv2_step_free(gsl_odeiv2_step *s);
#ifdef __cplusplus
}
#endif
#endif
