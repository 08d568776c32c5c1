/* TEST INFRASTRUCTURE — stand-in for the GSL error constants referenced. */
#pragma once
#define GSL_SUCCESS 0
#define GSL_EDOM 1
typedef void gsl_error_handler_t(const char*, const char*, int, int);
gsl_error_handler_t* gsl_set_error_handler_off(void);
