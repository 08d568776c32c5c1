/* TEST INFRASTRUCTURE — stand-in for gsl_sf_lnbeta. */
#pragma once
double gsl_sf_lnbeta(double a, double b);
