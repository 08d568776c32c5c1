// oracle_rng.h — TEST INFRASTRUCTURE (oracle), not product code.
//
// The draw stream shared by the oracle, the stand-in GSL used to build the
// reference for pinning, and the GPU sampler.  PhyloAcc-ST gives every
// element its own GSL generator seeded with the same SEED
// (src/PhyloAcc-ST/bpp_c.hpp:146-147) and draws from it sequentially through
// M0 -> M1 -> M2.  GSL is not available here, so the generator is replaced
// by a counter-based stream with the same structure:
//
//   word(w)    = Philox4x32-10( ctr = {w>>2 (low 32), w>>34, 0, 0},
//                               key = {SEED, 0} ) [w & 3]
//   uniform(w) = (word(w) + 0.5) * 2^-32            in (0, 1)
//
// Philox4x32-10 is the generator of Salmon, Moraes, Dror & Shaw, "Parallel
// random numbers: as easy as 1, 2, 3" (SC'11).  The samplers that consume
// the stream are written from their published definitions:
//   categorical (gsl_ran_multinomial with N = 1): inverse CDF on one uniform;
//   normal: Box-Muller (cosine branch), two uniforms;
//   gamma:  Marsaglia & Tsang (2000), "A simple method for generating gamma
//           variables", with the shape < 1 boost Gamma(a+1) * U^(1/a);
//   beta:   X / (X + Y), X ~ Gamma(a, 1) drawn before Y ~ Gamma(b, 1).
#pragma once
#include <cstdint>
#include <cmath>

namespace oracle_rng {

inline void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

struct Stream {
    uint32_t seed = 0;
    uint64_t pos = 0;           // index of the next word
    uint64_t cached_block = ~0ull;
    uint32_t cache[4] = {0, 0, 0, 0};

    void set(uint32_t s) { seed = s; pos = 0; cached_block = ~0ull; }

    uint32_t word_at(uint64_t w) {
        uint64_t b = w >> 2;
        if (b != cached_block) {
            uint32_t ctr[4] = {(uint32_t)b, (uint32_t)(b >> 32), 0u, 0u};
            uint32_t key[2] = {seed, 0u};
            philox4x32_10(ctr, key, cache);
            cached_block = b;
        }
        return cache[w & 3];
    }
    uint32_t next_word() { return word_at(pos++); }
    double uniform() { return ((double)next_word() + 0.5) * 2.3283064365386963e-10; }

    double normal() {
        double u1 = uniform();
        double u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }

    // Gamma with shape a and scale b.
    double gamma(double a, double b) {
        if (a < 1.0) {
            double g = gamma(a + 1.0, 1.0);
            double u = uniform();
            return b * g * std::pow(u, 1.0 / a);
        }
        double d = a - 1.0 / 3.0;
        double c = 1.0 / std::sqrt(9.0 * d);
        double x, v;
        for (;;) {
            do {
                x = normal();
                v = 1.0 + c * x;
            } while (v <= 0.0);
            v = v * v * v;
            double u = uniform();
            double x2 = x * x;
            if (u < 1.0 - 0.0331 * x2 * x2) break;
            if (std::log(u) < 0.5 * x2 + d * (1.0 - v + std::log(v))) break;
        }
        return b * d * v;
    }

    double beta(double a, double b) {
        double x = gamma(a, 1.0);
        double y = gamma(b, 1.0);
        return x / (x + y);
    }

    // Inverse-CDF categorical draw over unnormalised weights p[0..K-1].
    // Returns K if no weight is positive.
    int categorical(int K, const double* p) {
        double u = uniform();
        double total = 0;
        for (int k = 0; k < K; k++) total += p[k];
        double t = u * total;
        double cum = 0;
        for (int k = 0; k < K; k++) {
            cum += p[k];
            if (t < cum) return k;
        }
        for (int k = K - 1; k >= 0; k--)
            if (p[k] > 0) return k;
        return K;
    }
};

}  // namespace oracle_rng
