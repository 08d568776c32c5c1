// TEST INFRASTRUCTURE — implementations behind the stand-in GSL headers.
#include <cmath>
#include <cstdlib>

#include "gsl/gsl_errno.h"
#include "gsl/gsl_randist.h"
#include "gsl/gsl_rng.h"
#include "gsl/gsl_sf_gamma.h"
#include "oracle_rng.h"

static const gsl_rng_type shim_type = {"pacc-philox-stream"};
const gsl_rng_type* gsl_rng_default = &shim_type;

static oracle_rng::Stream* st(const gsl_rng* r) { return (oracle_rng::Stream*)r->state; }

gsl_rng* gsl_rng_alloc(const gsl_rng_type* T) {
    gsl_rng* r = new gsl_rng;
    r->type = T;
    r->state = new oracle_rng::Stream();
    st(r)->set(0);
    return r;
}
void gsl_rng_set(const gsl_rng* r, unsigned long int seed) { st(r)->set((uint32_t)seed); }
void gsl_rng_free(gsl_rng* r) {
    delete st(r);
    delete r;
}
double gsl_rng_uniform(const gsl_rng* r) { return st(r)->uniform(); }
double gsl_rng_uniform_pos(const gsl_rng* r) { return st(r)->uniform(); }

void gsl_ran_multinomial(const gsl_rng* r, size_t K, unsigned int N, const double p[], unsigned int n[]) {
    for (size_t k = 0; k < K; k++) n[k] = 0;
    for (unsigned int i = 0; i < N; i++) {
        int c = st(r)->categorical((int)K, p);
        if (c < (int)K) n[c]++;
    }
}
double gsl_ran_gamma(const gsl_rng* r, double a, double b) { return st(r)->gamma(a, b); }
double gsl_ran_gamma_pdf(double x, double a, double b) {
    if (x < 0) return 0.0;
    if (x == 0) return (a == 1) ? 1.0 / b : 0.0;
    return std::exp((a - 1) * std::log(x) - x / b - std::lgamma(a) - a * std::log(b));
}
double gsl_ran_beta(const gsl_rng* r, double a, double b) { return st(r)->beta(a, b); }
double gsl_ran_beta_pdf(double x, double a, double b) {
    if (x < 0 || x > 1) return 0.0;
    return std::exp((a - 1) * std::log(x) + (b - 1) * std::log1p(-x) - gsl_sf_lnbeta(a, b));
}
void gsl_ran_dirichlet(const gsl_rng* r, size_t K, const double alpha[], double theta[]) {
    double s = 0;
    for (size_t k = 0; k < K; k++) { theta[k] = st(r)->gamma(alpha[k], 1.0); s += theta[k]; }
    for (size_t k = 0; k < K; k++) theta[k] /= s;
}
double gsl_sf_lnbeta(double a, double b) { return std::lgamma(a) + std::lgamma(b) - std::lgamma(a + b); }
static void quiet_handler(const char*, const char*, int, int) {}
gsl_error_handler_t* gsl_set_error_handler_off(void) { return quiet_handler; }
