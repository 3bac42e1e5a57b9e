// gsl_shim.cpp -- definitions behind the GSL shim headers (test oracle only).
// The random-number generator is a Mersenne Twister (std::mt19937, the
// generator gsl_rng_mt19937 names); vectors are plain arrays; the
// minimisers, used only by the non-identity colour spaces, abort.
// gsl_shim_set_constant(v >= 0) makes every draw return v (the oracle's
// reproducible dither runs); v < 0 restores the Mersenne Twister.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <random>

#include <gsl/gsl_min.h>
#include <gsl/gsl_multimin.h>
#include <gsl/gsl_rng.h>
#include <gsl/gsl_vector.h>

[[noreturn]] static void gsl_shim_abort(const char* what)
{
    std::fprintf(stderr, "reference oracle: %s is not available\n", what);
    std::abort();
}

struct gsl_rng_s {
    std::mt19937 g;
};

static const gsl_rng_type mt_type = {"mt19937"};
const gsl_rng_type* gsl_rng_mt19937 = &mt_type;
unsigned long gsl_rng_default_seed = 0;

gsl_rng* gsl_rng_alloc(const gsl_rng_type*) { return new gsl_rng_s(); }
gsl_rng* gsl_rng_clone(const gsl_rng* r) { return new gsl_rng_s(*r); }
void gsl_rng_free(gsl_rng* r) { delete r; }
void gsl_rng_set(const gsl_rng* r, unsigned long s)
{
    const_cast<gsl_rng*>(r)->g.seed((uint32_t)(s == 0 ? 4357 : s));
}
static std::atomic<long long> g_constant_draw{-1};

extern "C" void gsl_shim_set_constant(long long value) { g_constant_draw.store(value); }

unsigned long gsl_rng_get(const gsl_rng* r)
{
    const long long c = g_constant_draw.load();
    return c >= 0 ? (unsigned long)(c & 0xffffffffLL) : (unsigned long)const_cast<gsl_rng*>(r)->g();
}
unsigned long gsl_rng_max(const gsl_rng*) { return 0xffffffffUL; }
unsigned long gsl_rng_min(const gsl_rng*) { return 0; }
double gsl_rng_uniform(const gsl_rng* r) { return gsl_rng_get(r) / 4294967296.0; }
unsigned long gsl_rng_uniform_int(const gsl_rng* r, unsigned long n) { return gsl_rng_get(r) % n; }

gsl_vector* gsl_vector_alloc(size_t n)
{
    gsl_vector* v = new gsl_vector();
    v->size = n;
    v->stride = 1;
    v->data = new double[n]();
    v->owner = 1;
    return v;
}
void gsl_vector_free(gsl_vector* v)
{
    if (v) {
        delete[] v->data;
        delete v;
    }
}
double gsl_vector_get(const gsl_vector* v, size_t i) { return v->data[i * v->stride]; }
void gsl_vector_set(gsl_vector* v, size_t i, double x) { v->data[i * v->stride] = x; }
void gsl_vector_set_all(gsl_vector* v, double x)
{
    for (size_t i = 0; i < v->size; ++i) v->data[i * v->stride] = x;
}
int gsl_vector_memcpy(gsl_vector* d, const gsl_vector* s)
{
    for (size_t i = 0; i < d->size && i < s->size; ++i) d->data[i * d->stride] = s->data[i * s->stride];
    return 0;
}

const gsl_min_fminimizer_type* gsl_min_fminimizer_brent = nullptr;
const gsl_min_fminimizer_type* gsl_min_fminimizer_goldensection = nullptr;
const gsl_min_fminimizer_type* gsl_min_fminimizer_quad_golden = nullptr;
gsl_min_fminimizer* gsl_min_fminimizer_alloc(const gsl_min_fminimizer_type*) { gsl_shim_abort("gsl_min_fminimizer_alloc"); }
void gsl_min_fminimizer_free(gsl_min_fminimizer*) {}
int gsl_min_fminimizer_set(gsl_min_fminimizer*, gsl_function*, double, double, double) { gsl_shim_abort("gsl_min"); }
int gsl_min_fminimizer_iterate(gsl_min_fminimizer*) { gsl_shim_abort("gsl_min"); }
double gsl_min_fminimizer_x_minimum(const gsl_min_fminimizer*) { gsl_shim_abort("gsl_min"); }
double gsl_min_fminimizer_x_lower(const gsl_min_fminimizer*) { gsl_shim_abort("gsl_min"); }
double gsl_min_fminimizer_x_upper(const gsl_min_fminimizer*) { gsl_shim_abort("gsl_min"); }
double gsl_min_fminimizer_f_minimum(const gsl_min_fminimizer*) { gsl_shim_abort("gsl_min"); }
const char* gsl_min_fminimizer_name(const gsl_min_fminimizer*) { return "shim"; }
int gsl_min_test_interval(double, double, double, double) { gsl_shim_abort("gsl_min"); }

const gsl_multimin_fminimizer_type* gsl_multimin_fminimizer_nmsimplex = nullptr;
const gsl_multimin_fminimizer_type* gsl_multimin_fminimizer_nmsimplex2 = nullptr;
const gsl_multimin_fminimizer_type* gsl_multimin_fminimizer_nmsimplex2rand = nullptr;
gsl_multimin_fminimizer* gsl_multimin_fminimizer_alloc(const gsl_multimin_fminimizer_type*, size_t)
{
    gsl_shim_abort("gsl_multimin_fminimizer_alloc");
}
void gsl_multimin_fminimizer_free(gsl_multimin_fminimizer*) {}
int gsl_multimin_fminimizer_set(gsl_multimin_fminimizer*, gsl_multimin_function*, const gsl_vector*, const gsl_vector*)
{
    gsl_shim_abort("gsl_multimin");
}
int gsl_multimin_fminimizer_iterate(gsl_multimin_fminimizer*) { gsl_shim_abort("gsl_multimin"); }
double gsl_multimin_fminimizer_minimum(const gsl_multimin_fminimizer*) { gsl_shim_abort("gsl_multimin"); }
double gsl_multimin_fminimizer_size(const gsl_multimin_fminimizer*) { gsl_shim_abort("gsl_multimin"); }
gsl_vector* gsl_multimin_fminimizer_x(const gsl_multimin_fminimizer*) { gsl_shim_abort("gsl_multimin"); }
const char* gsl_multimin_fminimizer_name(const gsl_multimin_fminimizer*) { return "shim"; }
int gsl_multimin_test_size(double, double) { gsl_shim_abort("gsl_multimin"); }
