/* orc_internal.h -- shared declarations inside the oracle (test infrastructure only). */
#ifndef ORC_INTERNAL_H
#define ORC_INTERNAL_H

typedef void (*orc_rhs)(double t, const double *y, double *dydt, void *p);

/* one accepted adaptive step towards t1; returns 0 on success */
int orc_evolve_apply(orc_rhs rhs, void *p, double *t, double t1, double *h, double *y,
                     double epsabs, double epsrel);

extern _Thread_local long long orc_brent_iterations;

typedef struct orc_brent {
    double (*f)(double, void *);
    void *p;
    double a, b, c, fa, fb, fc, d, e;
    double root, lo, hi;
} orc_brent;

void orc_brent_init(orc_brent *s, double (*f)(double, void *), void *p, double lo, double hi,
                    double flo, double fhi);
void orc_brent_step(orc_brent *s);
int orc_root_test_interval(double lo, double hi, double epsabs, double epsrel);

#endif
