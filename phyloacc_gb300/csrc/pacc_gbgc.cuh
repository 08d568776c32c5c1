// pacc_gbgc.cuh — device helpers of the gBGC model shared by its likelihood
// engine (pacc_gbgc.cu) and its chain kernel (pacc_gbgc_chain.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pacc {

// getRate (bpp_c.cpp:13-30): Q0 scaled entrywise by f(s + b B_ij) with
// f(x) = x / (1 - e^-x) (f(0) = 1), B_ij = +1 from A/T to C/G, -1 from C/G
// to A/T, 0 otherwise (the diagonal included); then each diagonal entry
// reset so that its row sums to zero.
static __device__ void gbgc_rate(const double* Q0, double s, double b, double* Q) {
    for (int q = 0; q < 16; q++) Q[q] = Q0[q];
    if (s == 0 && b == 0) return;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            const bool weak_i = (i == 0 || i == 3), weak_j = (j == 0 || j == 3);
            const double bij = (weak_i && !weak_j) ? b : ((!weak_i && weak_j) ? -b : 0.0);
            const double v = bij + s;
            Q[i * 4 + j] *= (v == 0) ? 1.0 : v / (1 - exp(-v));
        }
    for (int i = 0; i < 4; i++) {
        double c = 0;
        for (int j = 0; j < 4; j++) c += Q[i * 4 + j];
        Q[i * 4 + i] -= c;
    }
}

// Exact power-of-two rescaling of linear partials in FP32 or FP64.
template <typename Real> struct GbgcScale;
template <> struct GbgcScale<float> {
    static __device__ __forceinline__ float tiny() { return 0x1p-60f; }
    static __device__ __forceinline__ float pow2(int k) { return ldexpf(1.0f, k); }
    static __device__ __forceinline__ int expo(float x) { int e; frexpf(x, &e); return e; }
};
template <> struct GbgcScale<double> {
    static __device__ __forceinline__ double tiny() { return 0x1p-500; }
    static __device__ __forceinline__ double pow2(int k) { return ldexp(1.0, k); }
    static __device__ __forceinline__ int expo(double x) { int e; frexp(x, &e); return e; }
};

// m(j) = sum_i P[i][j] L(i): what a child sends its parent (log_multi,
// bpp.hpp:414-431, in linear space)
template <typename Real>
__device__ __forceinline__ void gbgc_message(const Real* P, const Real* L, Real* m) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
        Real v = P[j] * L[0];
        v = fma(P[4 + j], L[1], v);
        v = fma(P[8 + j], L[2], v);
        v = fma(P[12 + j], L[3], v);
        m[j] = v;
    }
}

}  // namespace pacc
