/* GSL stand-in (test infrastructure): gsl_function and GSL_FN_EVAL. */
#ifndef FJREF_GSL_MATH_H
#define FJREF_GSL_MATH_H
#include <math.h>
#ifdef __cplusplus
extern "C" {
#endif
struct gsl_function_struct {
    double (*function)(double x, void *params);
    void *params;
};
typedef struct gsl_function_struct gsl_function;
#define GSL_FN_EVAL(F, x) (*((F)->function))(x, (F)->params)
#ifdef __cplusplus
}
#endif
#endif
