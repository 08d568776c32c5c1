/* TEST INFRASTRUCTURE — stand-in for the GSL random-variate API used by
 * PhyloAcc-ST; the samplers are the published methods of oracle/oracle_rng.h. */
#pragma once
#include <stddef.h>
#include "gsl_rng.h"
void gsl_ran_multinomial(const gsl_rng* r, size_t K, unsigned int N, const double p[], unsigned int n[]);
double gsl_ran_gamma(const gsl_rng* r, double a, double b);
double gsl_ran_gamma_pdf(double x, double a, double b);
double gsl_ran_beta(const gsl_rng* r, double a, double b);
double gsl_ran_beta_pdf(double x, double a, double b);
void gsl_ran_dirichlet(const gsl_rng* r, size_t K, const double alpha[], double theta[]);
