/* Minimal GSL random-number interface for the reference's mersenne.h (test
 * oracle only): a Mersenne-Twister generator on std::mt19937, as
 * gsl_rng_mt19937 (the oracle compares the pre-dither levels, not draws). */
#ifndef ENB_REFSHIM_GSL_RNG_H
#define ENB_REFSHIM_GSL_RNG_H

typedef struct gsl_rng_type_s { const char* name; } gsl_rng_type;
typedef struct gsl_rng_s gsl_rng;

extern const gsl_rng_type* gsl_rng_mt19937;
extern unsigned long gsl_rng_default_seed;
gsl_rng* gsl_rng_alloc(const gsl_rng_type*);
gsl_rng* gsl_rng_clone(const gsl_rng*);
void gsl_rng_free(gsl_rng*);
void gsl_rng_set(const gsl_rng*, unsigned long);
unsigned long gsl_rng_get(const gsl_rng*);
double gsl_rng_uniform(const gsl_rng*);
unsigned long gsl_rng_uniform_int(const gsl_rng*, unsigned long);
unsigned long gsl_rng_max(const gsl_rng*);
unsigned long gsl_rng_min(const gsl_rng*);

#endif
