/* Minimal GSL vector declarations (test oracle only). */
#ifndef ENB_REFSHIM_GSL_VECTOR_H
#define ENB_REFSHIM_GSL_VECTOR_H
#include <cstddef>
typedef struct { size_t size; size_t stride; double* data; void* block; int owner; } gsl_vector;
gsl_vector* gsl_vector_alloc(size_t);
void gsl_vector_free(gsl_vector*);
double gsl_vector_get(const gsl_vector*, size_t);
void gsl_vector_set(gsl_vector*, size_t, double);
void gsl_vector_set_all(gsl_vector*, double);
int gsl_vector_memcpy(gsl_vector*, const gsl_vector*);
#endif
