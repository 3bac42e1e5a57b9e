/* Minimal GSL multidimensional minimiser declarations (test oracle only). */
#ifndef ENB_REFSHIM_GSL_MULTIMIN_H
#define ENB_REFSHIM_GSL_MULTIMIN_H
#include <cstddef>
#include <gsl/gsl_errno.h>
#include <gsl/gsl_vector.h>
typedef struct { double (*f)(const gsl_vector*, void*); size_t n; void* params; } gsl_multimin_function;
typedef struct gsl_multimin_fminimizer_type_s { const char* name; } gsl_multimin_fminimizer_type;
typedef struct gsl_multimin_fminimizer_s { const gsl_multimin_fminimizer_type* type; gsl_vector* x; double fval; double size; } gsl_multimin_fminimizer;
extern const gsl_multimin_fminimizer_type* gsl_multimin_fminimizer_nmsimplex;
extern const gsl_multimin_fminimizer_type* gsl_multimin_fminimizer_nmsimplex2;
extern const gsl_multimin_fminimizer_type* gsl_multimin_fminimizer_nmsimplex2rand;
gsl_multimin_fminimizer* gsl_multimin_fminimizer_alloc(const gsl_multimin_fminimizer_type*, size_t);
void gsl_multimin_fminimizer_free(gsl_multimin_fminimizer*);
int gsl_multimin_fminimizer_set(gsl_multimin_fminimizer*, gsl_multimin_function*, const gsl_vector*, const gsl_vector*);
int gsl_multimin_fminimizer_iterate(gsl_multimin_fminimizer*);
double gsl_multimin_fminimizer_minimum(const gsl_multimin_fminimizer*);
double gsl_multimin_fminimizer_size(const gsl_multimin_fminimizer*);
gsl_vector* gsl_multimin_fminimizer_x(const gsl_multimin_fminimizer*);
const char* gsl_multimin_fminimizer_name(const gsl_multimin_fminimizer*);
int gsl_multimin_test_size(double, double);
#endif
