/*
 * gsl_standin.c -- project-written stand-in for the GSL subset the reference
 * calls (GSL itself is absent from this machine).  TEST INFRASTRUCTURE ONLY:
 * it lets the reference's own sources compile, unmodified, into oracle/_ref.
 * The algorithms are the oracle's restatements of the published methods
 * (orc_numerics.c): Brent steps, QUADPACK QAGS/QAGIU and the RK8(7) pair of
 * Prince & Dormand (the method gsl_odeiv2_step_rk8pd names) under GSL's
 * documented y-error step control.
 */
#include <stdlib.h>
#include "gsl/gsl_errno.h"
#include "gsl/gsl_integration.h"
#include "gsl/gsl_odeiv2.h"
#include "gsl/gsl_roots.h"
#include "../fjoracle.h"
#include "../orc_internal.h"

gsl_error_handler_t *gsl_set_error_handler_off(void) { return NULL; }

/* ---- roots ---- */
struct fjref_root_type { int unused; };
static const struct fjref_root_type brent_type = {0};
const gsl_root_fsolver_type *gsl_root_fsolver_brent = &brent_type;
struct fjref_root_solver { gsl_function fn; orc_brent st; };

static double call_fn(double x, void *p)
{
    gsl_function *F = (gsl_function *)p;
    return GSL_FN_EVAL(F, x);
}
gsl_root_fsolver *gsl_root_fsolver_alloc(const gsl_root_fsolver_type *T)
{
    (void)T;
    return (gsl_root_fsolver *)calloc(1, sizeof(gsl_root_fsolver));
}
int gsl_root_fsolver_set(gsl_root_fsolver *s, gsl_function *f, double lo, double hi)
{
    s->fn = *f;
    orc_brent_init(&s->st, call_fn, &s->fn, lo, hi, call_fn(lo, &s->fn), call_fn(hi, &s->fn));
    return GSL_SUCCESS;
}
int gsl_root_fsolver_iterate(gsl_root_fsolver *s) { orc_brent_step(&s->st); return GSL_SUCCESS; }
double gsl_root_fsolver_root(const gsl_root_fsolver *s) { return s->st.root; }
double gsl_root_fsolver_x_lower(const gsl_root_fsolver *s) { return s->st.lo; }
double gsl_root_fsolver_x_upper(const gsl_root_fsolver *s) { return s->st.hi; }
void gsl_root_fsolver_free(gsl_root_fsolver *s) { free(s); }
int gsl_root_test_interval(double lo, double hi, double epsabs, double epsrel)
{
    return orc_root_test_interval(lo, hi, epsabs, epsrel) ? GSL_SUCCESS : GSL_CONTINUE;
}

/* ---- integration ---- */
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n)
{
    gsl_integration_workspace *w = (gsl_integration_workspace *)malloc(sizeof *w);
    w->limit = n;
    return w;
}
void gsl_integration_workspace_free(gsl_integration_workspace *w) { free(w); }
int gsl_integration_qags(const gsl_function *f, double a, double b, double epsabs, double epsrel,
                         size_t limit, gsl_integration_workspace *w, double *result, double *abserr)
{
    (void)w;
    gsl_function F = *f;
    return orc_qags(call_fn, &F, a, b, epsabs, epsrel, (int)limit, result, abserr);
}
int gsl_integration_qagiu(gsl_function *f, double a, double epsabs, double epsrel, size_t limit,
                          gsl_integration_workspace *w, double *result, double *abserr)
{
    (void)w;
    return orc_qagiu(call_fn, f, a, epsabs, epsrel, (int)limit, result, abserr);
}

/* ---- ODE ---- */
struct fjref_step_type { int unused; };
static const struct fjref_step_type rk_type = {0};
const gsl_odeiv2_step_type *gsl_odeiv2_step_rk8pd = &rk_type;
struct fjref_step { int dim; };
struct fjref_control { double epsabs, epsrel; };
struct fjref_evolve { int dim; };

gsl_odeiv2_step *gsl_odeiv2_step_alloc(const gsl_odeiv2_step_type *T, size_t dim)
{
    (void)T;
    gsl_odeiv2_step *s = (gsl_odeiv2_step *)malloc(sizeof *s);
    s->dim = (int)dim;
    return s;
}
gsl_odeiv2_control *gsl_odeiv2_control_y_new(double eps_abs, double eps_rel)
{
    gsl_odeiv2_control *c = (gsl_odeiv2_control *)malloc(sizeof *c);
    c->epsabs = eps_abs;
    c->epsrel = eps_rel;
    return c;
}
gsl_odeiv2_evolve *gsl_odeiv2_evolve_alloc(size_t dim)
{
    gsl_odeiv2_evolve *e = (gsl_odeiv2_evolve *)malloc(sizeof *e);
    e->dim = (int)dim;
    return e;
}
static void rhs_adapt(double t, const double *y, double *dydt, void *p)
{
    const gsl_odeiv2_system *sys = (const gsl_odeiv2_system *)p;
    sys->function(t, y, dydt, sys->params);
}
int gsl_odeiv2_evolve_apply(gsl_odeiv2_evolve *e, gsl_odeiv2_control *con, gsl_odeiv2_step *step,
                            const gsl_odeiv2_system *sys, double *t, double t1, double *h, double y[])
{
    (void)e; (void)step;
    return orc_evolve_apply(rhs_adapt, (void *)sys, t, t1, h, y, con->epsabs, con->epsrel);
}
void gsl_odeiv2_evolve_free(gsl_odeiv2_evolve *e) { free(e); }
void gsl_odeiv2_control_free(gsl_odeiv2_control *c) { free(c); }
void gsl_odeiv2_step_free(gsl_odeiv2_step *s) { free(s); }
