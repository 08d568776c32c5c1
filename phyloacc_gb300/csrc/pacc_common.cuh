// pacc_common.cuh — device helpers shared by the chain kernels.
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "pacc_dev.h"
#include "pacc_rng.cuh"

namespace pacc {

// Model constants; every translation unit that includes this header holds its
// own copy, filled by that unit's set_model function.
static __constant__ DevModel dM;

// Gamma(shape a, scale b) density and its log as the reference takes it (bpp_c.cpp:784,1046).
static __device__ __noinline__ double gamma_pdf(double x, double a, double b) {
    if (x < 0) return 0.0;
    if (x == 0) return (a == 1) ? 1.0 / b : 0.0;
    double t = __dsub_rn(__dsub_rn(__dsub_rn(__dmul_rn(a - 1, d_log(x)), __ddiv_rn(x, b)), d_lgamma(a)),
                         __dmul_rn(a, d_log(b)));
    return d_exp(t);
}
static __device__ __forceinline__ double log_gamma_pdf(double x, double a, double b) { return d_log(gamma_pdf(x, a, b)); }
static __device__ __forceinline__ double lnbeta(double a, double b) {
    return __dsub_rn(__dadd_rn(d_lgamma(a), d_lgamma(b)), d_lgamma(__dadd_rn(a, b)));
}

// P^T(d*r) = eigeninv * diag(exp(lambda*d*r)) * eigenvec  (bpp.hpp:375-380), FP64.
// scaled=false uses exp(lambda*d) as the null-rate cache does (bpp.hpp:375).
static __device__ __noinline__ void build_pt(double d, double r, bool scaled, double* out) {
    double e[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        double x = __dmul_rn(dM.lam[i], d);
        if (scaled) x = __dmul_rn(x, r);
        e[i] = d_exp(x);
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
            double s = 0;
#pragma unroll
            for (int i = 0; i < 4; i++) s = __dadd_rn(s, __dmul_rn(dM.einv[a * 4 + i], __dmul_rn(dM.evec[i * 4 + b], e[i])));
            out[a * 4 + b] = s;
        }
}

static __device__ void identity_pt(double* out) {
#pragma unroll
    for (int a = 0; a < 16; a++) out[a] = ((a >> 2) == (a & 3)) ? 1.0 : 0.0;
}

static __device__ __forceinline__ uint64_t fnv_step(uint64_t h, uint8_t b) {
    return (h ^ b) * 0x100000001b3ull;
}

}  // namespace pacc
