/* Minimal GSL one-dimensional minimiser declarations (test oracle only;
 * the minimisers serve only the non-identity colour spaces). */
#ifndef ENB_REFSHIM_GSL_MIN_H
#define ENB_REFSHIM_GSL_MIN_H
#include <math.h>
#include <gsl/gsl_errno.h>
typedef struct { double (*function)(double, void*); void* params; } gsl_function;
typedef struct gsl_min_fminimizer_type_s { const char* name; } gsl_min_fminimizer_type;
typedef struct gsl_min_fminimizer_s gsl_min_fminimizer;
extern const gsl_min_fminimizer_type* gsl_min_fminimizer_brent;
extern const gsl_min_fminimizer_type* gsl_min_fminimizer_goldensection;
extern const gsl_min_fminimizer_type* gsl_min_fminimizer_quad_golden;
gsl_min_fminimizer* gsl_min_fminimizer_alloc(const gsl_min_fminimizer_type*);
void gsl_min_fminimizer_free(gsl_min_fminimizer*);
int gsl_min_fminimizer_set(gsl_min_fminimizer*, gsl_function*, double, double, double);
int gsl_min_fminimizer_iterate(gsl_min_fminimizer*);
double gsl_min_fminimizer_x_minimum(const gsl_min_fminimizer*);
double gsl_min_fminimizer_x_lower(const gsl_min_fminimizer*);
double gsl_min_fminimizer_x_upper(const gsl_min_fminimizer*);
double gsl_min_fminimizer_f_minimum(const gsl_min_fminimizer*);
const char* gsl_min_fminimizer_name(const gsl_min_fminimizer*);
int gsl_min_test_interval(double, double, double, double);
#endif
