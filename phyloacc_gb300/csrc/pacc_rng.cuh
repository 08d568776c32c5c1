// pacc_rng.cuh — the element draw stream on the device.
//
// PhyloAcc-ST draws every random number of an element from one generator
// seeded with SEED (src/PhyloAcc-ST/bpp_c.hpp:146-147), sequentially through
// M0, M1 and M2.  The GPU keeps that structure with a counter-based stream, so
// any draw can be generated from its position alone:
//   word(w)    = Philox4x32-10(ctr = {w>>2, w>>34, 0, 0}, key = {SEED, 0})[w & 3]
//   uniform(w) = (word(w) + 0.5) * 2^-32
// (Salmon, Moraes, Dror & Shaw, SC'11).  Columns of the internal-base pass
// take their words at static per-column offsets (a prefix sum of the draws
// each column makes), so columns are sampled in parallel while consuming the
// stream exactly as the sequential loop of bpp_c.cpp:382-383 does.
//
// Samplers (one thread, sequential positions): categorical by inverse CDF on
// one uniform; normal by Box-Muller (cosine branch); gamma by Marsaglia &
// Tsang (2000) with the Gamma(a+1) U^(1/a) boost for a < 1; beta as
// X/(X+Y).  Scalar arithmetic uses explicitly rounded operations (no FMA
// contraction) so that it rounds like the host build of the same formulas.
#pragma once
#include <stdint.h>

namespace pacc {

// Out-of-line math: the chain's scalar code calls these from many places, and
// one copy of each library routine (instead of one inlined per call site)
// keeps the kernels small enough for the instruction caches.  The values are
// those of the library functions they wrap.
static __device__ __noinline__ double d_log(double x) { return log(x); }
static __device__ __noinline__ double d_exp(double x) { return exp(x); }
static __device__ __noinline__ double d_pow(double x, double y) { return pow(x, y); }
static __device__ __noinline__ double d_lgamma(double x) { return lgamma(x); }
static __device__ __noinline__ double d_cos(double x) { return cos(x); }
static __device__ __noinline__ float f_log(float x) { return logf(x); }

__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                              uint32_t k1, uint32_t out[4]) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

__device__ __forceinline__ double word_to_uniform(uint32_t w) {
    return __dmul_rn((double)w + 0.5, 2.3283064365386963e-10);
}

// Sequential reader with a one-block cache.
struct StreamReader {
    uint32_t seed;
    uint64_t pos;
    uint64_t blk;
    uint32_t cache[4];
    __device__ void init(uint32_t s, uint64_t p) { seed = s; pos = p; blk = ~0ull; }
    __device__ uint32_t word_at(uint64_t w) {
        uint64_t b = w >> 2;
        if (b != blk) {
            philox4x32_10((uint32_t)b, (uint32_t)(b >> 32), 0u, 0u, seed, 0u, cache);
            blk = b;
        }
        return cache[w & 3];
    }
    __device__ double uniform() { return word_to_uniform(word_at(pos++)); }
    __device__ __noinline__ double normal() {
        double u1 = uniform();
        double u2 = uniform();
        return __dmul_rn(__dsqrt_rn(__dmul_rn(-2.0, d_log(u1))), d_cos(__dmul_rn(6.283185307179586, u2)));
    }
    __device__ __noinline__ double gamma(double a, double b) {
        if (a < 1.0) {
            double g = gamma_ge1(__dadd_rn(a, 1.0), 1.0);
            double u = uniform();
            return __dmul_rn(__dmul_rn(b, g), d_pow(u, __ddiv_rn(1.0, a)));
        }
        return gamma_ge1(a, b);
    }
    // Marsaglia-Tsang for shape >= 1; returns (b*d)*v.
    __device__ __noinline__ double gamma_ge1(double a, double b) {
        double d = __dsub_rn(a, 1.0 / 3.0);
        double c = __ddiv_rn(1.0, __dsqrt_rn(__dmul_rn(9.0, d)));
        double x, v;
        for (int guard = 0; guard < 100000; guard++) {
            do {
                x = normal();
                v = __dadd_rn(1.0, __dmul_rn(c, x));
            } while (v <= 0.0);
            v = __dmul_rn(__dmul_rn(v, v), v);
            double u = uniform();
            double x2 = __dmul_rn(x, x);
            if (u < __dsub_rn(1.0, __dmul_rn(__dmul_rn(0.0331, x2), x2))) break;
            if (d_log(u) < __dadd_rn(__dmul_rn(0.5, x2), __dmul_rn(d, __dadd_rn(__dsub_rn(1.0, v), d_log(v))))) break;
        }
        return __dmul_rn(__dmul_rn(b, d), v);
    }
    __device__ __noinline__ double beta(double a, double b) {
        double x = gamma(a, 1.0);
        double y = gamma(b, 1.0);
        return __ddiv_rn(x, __dadd_rn(x, y));
    }
};

// The same samplers in FP32 arithmetic, for the FP32-partial path (its
// rate proposals and transition-rate draws; the MH ratio stays FP64).
// Uniforms take the top 24 bits of a word: ((w >> 8) + 0.5) * 2^-24.
struct StreamReader32 {
    uint32_t seed;
    uint64_t pos;
    uint64_t blk;
    uint32_t cache[4];
    __device__ void init(uint32_t s, uint64_t p) { seed = s; pos = p; blk = ~0ull; }
    __device__ uint32_t word_at(uint64_t w) {
        const uint64_t b = w >> 2;
        if (b != blk) {
            philox4x32_10((uint32_t)b, (uint32_t)(b >> 32), 0u, 0u, seed, 0u, cache);
            blk = b;
        }
        return cache[w & 3];
    }
    __device__ float uniform() { return ((float)(word_at(pos++) >> 8) + 0.5f) * 5.9604644775390625e-08f; }
    __device__ float normal() {
        const float u1 = uniform();
        const float u2 = uniform();
        return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
    }
    // Marsaglia-Tsang for shape >= 1; returns (b*d)*v.
    __device__ float gamma_ge1(float a, float b) {
        const float d = a - 1.0f / 3.0f;
        const float c = 1.0f / sqrtf(9.0f * d);
        float x, v;
        for (int guard = 0; guard < 100000; guard++) {
            do {
                x = normal();
                v = 1.0f + c * x;
            } while (v <= 0.0f);
            v = v * v * v;
            const float u = uniform();
            const float x2 = x * x;
            if (u < 1.0f - 0.0331f * x2 * x2) break;
            if (logf(u) < 0.5f * x2 + d * (1.0f - v + logf(v))) break;
        }
        return b * d * v;
    }
    __device__ __noinline__ float gamma(float a, float b) {
        if (a < 1.0f) {
            const float g = gamma_ge1(a + 1.0f, 1.0f);
            const float u = uniform();
            return b * g * powf(u, 1.0f / a);
        }
        return gamma_ge1(a, b);
    }
    __device__ float beta(float a, float b) {
        const float x = gamma(a, 1.0f);
        const float y = gamma(b, 1.0f);
        return x / (x + y);
    }
};

// Inverse-CDF categorical draw over K unnormalised weights (K <= 4).
template <typename T>
__device__ __forceinline__ int categorical(int K, const T* p, double u) {
    double total = 0;
    for (int k = 0; k < K; k++) total = __dadd_rn(total, (double)p[k]);
    double t = __dmul_rn(u, total);
    double cum = 0;
    for (int k = 0; k < K; k++) {
        cum = __dadd_rn(cum, (double)p[k]);
        if (t < cum) return k;
    }
    for (int k = K - 1; k >= 0; k--)
        if (p[k] > 0) return k;
    return K;
}

}  // namespace pacc
