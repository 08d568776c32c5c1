/* TEST INFRASTRUCTURE — stand-in for the GSL generator API used by
 * PhyloAcc-ST (gsl_rng_alloc/set/free/uniform).  The generator behind it is
 * the counter-based stream of oracle/oracle_rng.h, not mt19937. */
#pragma once
#include <stdint.h>
typedef struct gsl_rng_type { const char* name; } gsl_rng_type;
typedef struct gsl_rng { const gsl_rng_type* type; void* state; } gsl_rng;
extern const gsl_rng_type* gsl_rng_default;
gsl_rng* gsl_rng_alloc(const gsl_rng_type* T);
void gsl_rng_set(const gsl_rng* r, unsigned long int seed);
void gsl_rng_free(gsl_rng* r);
double gsl_rng_uniform(const gsl_rng* r);
double gsl_rng_uniform_pos(const gsl_rng* r);
