// pacc_gbgc.cu — the likelihood engine of the PhyloAcc-ST-GBGC model on the
// GPU (sm_103a): per-branch transition matrices of the rate matrix under
// selection and GC-biased gene conversion, the pruning pass and the
// expected-count pass over one element's columns.
//
// The reference (src/PhyloAcc-ST-GBGC/SRC) keeps six classes of branch
// matrices, chosen by 2 Z + B in Update_Tg (bpp_c.cpp:494-517), built from
// Q(s, b) = getRate(Q0, s, b) (bpp_c.cpp:13-30) by one eigendecomposition per
// class (init_cache_TM, bpp_c.cpp:1563-1621).  Here every (class, branch)
// exponential exp(Q(s, b) d) is a Padé [13/13] approximant with scaling and
// squaring (Higham, "The scaling and squaring method for the matrix
// exponential revisited", SIAM J. Matrix Anal. Appl. 26(4), 2005), in FP64,
// one thread per matrix: no eigensystem per class, and no loss where one
// would be ill-conditioned.  Matrices are stored transposed, P[child][parent],
// as the reference's cache holds them.
//
// The passes run one column per lane.  Partials are linear (FP32 or FP64)
// with exact power-of-two rescaling and an integer exponent per node and
// column; the column log-likelihood is formed in FP64.  The expected counts
// of the sampling pass (bpp_c.cpp:541-596) are the joint posteriors
//   P(child i, parent j | column) = q_parent(j) P[i][j] L_child(i) / m_child(j)
// with m_child(j) = sum_i P[i][j] L_child(i) the child's message: reduced
// over a warp's 32 columns with shuffles in a fixed order, added to the
// warp's own slice of per-warp sums, and the slices summed in warp order, so
// the counts do not depend on timing.
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "pacc_dev.h"
#include "pacc_gbgc.cuh"

namespace pacc {

__device__ __forceinline__ void mm4(const double* A, const double* B, double* C) {
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            double s = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) s = fma(A[i * 4 + k], B[k * 4 + j], s);
            C[i * 4 + j] = s;
        }
}

// exp(A) of a 4x4 FP64 matrix: Padé [13/13] approximant of A / 2^sq, then sq
// squarings; sq the least with ||A||_1 / 2^sq <= theta_13.
__device__ void expm4(const double* A0, double* E) {
    const double b[14] = {64764752532480000.0, 32382376266240000.0, 7771770303897600.0, 1187353796428800.0,
                          129060195264000.0,   10559470521600.0,    670442572800.0,    33522128640.0,
                          1323241920.0,        40840800.0,          960960.0,          16380.0,
                          182.0,               1.0};
    const double theta13 = 5.371920351148152;
    double nrm = 0;
    for (int j = 0; j < 4; j++) {
        double c = 0;
        for (int i = 0; i < 4; i++) c += fabs(A0[i * 4 + j]);
        nrm = fmax(nrm, c);
    }
    int sq = 0;
    if (nrm > theta13) sq = (int)ceil(log2(nrm / theta13));
    const double f = ldexp(1.0, -sq);
    double A[16], A2[16], A4[16], A6[16], T[16], U[16], V[16];
    for (int q = 0; q < 16; q++) A[q] = A0[q] * f;
    mm4(A, A, A2);
    mm4(A2, A2, A4);
    mm4(A4, A2, A6);
    // U = A [A6 (b13 A6 + b11 A4 + b9 A2) + b7 A6 + b5 A4 + b3 A2 + b1 I]
    for (int q = 0; q < 16; q++) T[q] = b[13] * A6[q] + b[11] * A4[q] + b[9] * A2[q];
    mm4(A6, T, V);
    for (int q = 0; q < 16; q++) {
        V[q] += b[7] * A6[q] + b[5] * A4[q] + b[3] * A2[q];
        if (q % 5 == 0) V[q] += b[1];
    }
    mm4(A, V, U);
    // V = A6 (b12 A6 + b10 A4 + b8 A2) + b6 A6 + b4 A4 + b2 A2 + b0 I
    for (int q = 0; q < 16; q++) T[q] = b[12] * A6[q] + b[10] * A4[q] + b[8] * A2[q];
    mm4(A6, T, V);
    for (int q = 0; q < 16; q++) {
        V[q] += b[6] * A6[q] + b[4] * A4[q] + b[2] * A2[q];
        if (q % 5 == 0) V[q] += b[0];
    }
    // (V - U) E = (V + U): Gaussian elimination with partial pivoting
    double M[16], R[16];
    for (int q = 0; q < 16; q++) { M[q] = V[q] - U[q]; R[q] = V[q] + U[q]; }
    for (int k = 0; k < 4; k++) {
        int pr = k;
        for (int i = k + 1; i < 4; i++)
            if (fabs(M[i * 4 + k]) > fabs(M[pr * 4 + k])) pr = i;
        if (pr != k)
            for (int j = 0; j < 4; j++) {
                double t = M[k * 4 + j]; M[k * 4 + j] = M[pr * 4 + j]; M[pr * 4 + j] = t;
                t = R[k * 4 + j]; R[k * 4 + j] = R[pr * 4 + j]; R[pr * 4 + j] = t;
            }
        for (int i = k + 1; i < 4; i++) {
            const double l = M[i * 4 + k] / M[k * 4 + k];
            for (int j = k; j < 4; j++) M[i * 4 + j] -= l * M[k * 4 + j];
            for (int j = 0; j < 4; j++) R[i * 4 + j] -= l * R[k * 4 + j];
        }
    }
    for (int k = 3; k >= 0; k--)
        for (int j = 0; j < 4; j++) {
            double s = R[k * 4 + j];
            for (int c = k + 1; c < 4; c++) s -= M[k * 4 + c] * E[c * 4 + j];
            E[k * 4 + j] = s / M[k * 4 + k];
        }
    for (int r = 0; r < sq; r++) {
        mm4(E, E, T);
        for (int q = 0; q < 16; q++) E[q] = T[q];
    }
}

// One thread per (class, branch): P = exp(Q_class d)^T for every branch of
// the element's tree that is not missing.  The accelerated classes are not
// built on the outgroup path, which init_cache_TM leaves at zero as well.
template <typename Real>
__global__ void gbgc_pmat_kernel(GbgcParams p) {
    const int nb = p.n_nodes - 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 6 * nb) return;
    const int k = t / nb, s = p.nodes[t % nb];
    if (p.missing[s] || ((k == 2 || k == 5) && p.fixed[s])) return;
    const double sel = (k % 3 == 1) ? p.sc : ((k % 3 == 2) ? p.sn : 0.0);
    const double bias = k >= 3 ? p.gb : 0.0;
    double Q[16], A[16], E[16];
    gbgc_rate(p.Q0, sel, bias, Q);
    for (int q = 0; q < 16; q++) A[q] = Q[q] * p.dist[s];
    expm4(A, E);
    Real* pm = (Real*)p.pmat;
    for (int q = 0; q < 16; q++) {
        const double v = E[(q & 3) * 4 + (q >> 2)];   // (child q/4, parent q%4) = E[parent][child]
        p.logp[((size_t)k * p.N + s) * 16 + q] = log(v);
        pm[((size_t)k * p.N + s) * 16 + q] = (Real)v;
    }
}

// A node's partial at column g: a leaf's allowed bases, or an internal node's
// stored partial and exponent.
template <typename Real>
__device__ __forceinline__ void gbgc_load(const GbgcParams& p, int s, int g, Real* L, int* e) {
    if (s < p.S) {
        const int msk = p.masks[(size_t)s * p.GGp + g];
#pragma unroll
        for (int i = 0; i < 4; i++) L[i] = ((msk >> i) & 1) ? Real(1) : Real(0);
        *e = 0;
    } else {
        const Real* q = (const Real*)p.part + ((size_t)s * p.GGp + g) * 4;
#pragma unroll
        for (int i = 0; i < 4; i++) L[i] = q[i];
        *e = p.scl[(size_t)s * p.GGp + g];
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One CTA of p.warps warps; lane l of warp w takes columns w*32 + l + k*32*warps.
template <typename Real>
__global__ void gbgc_engine_kernel(GbgcParams p) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const Real* pm = (const Real*)p.pmat;
    Real* part = (Real*)p.part;
    double* wc = p.wcounts + (size_t)w * p.N * 16;
    for (int i = lane; i < p.N * 16; i += 32) wc[i] = 0;
    __syncwarp();
    for (int g0 = w * 32; g0 < p.GGp; g0 += p.warps * 32) {
        const int g = g0 + lane;
        const bool real_col = g < p.GG;
        // pruning pass (bpp_c.cpp:480-515): partials of the internal nodes in postorder
        for (int k = 0; k < p.n_nodes; k++) {
            const int s = p.nodes[k];
            if (s < p.S || p.missing[s]) continue;
            Real a[4] = {1, 1, 1, 1};
            int e = 0;
            const int ch[2] = {p.c0[s], p.c1[s]};
            for (int q = 0; q < 2; q++) {
                const int c = ch[q];
                if (p.missing[c]) continue;
                Real L[4], m[4];
                int ec;
                gbgc_load(p, c, g, L, &ec);
                gbgc_message(pm + ((size_t)p.cls[c] * p.N + c) * 16, L, m);
#pragma unroll
                for (int j = 0; j < 4; j++) a[j] *= m[j];
                e += ec;
            }
            const Real mx = fmax(fmax(a[0], a[1]), fmax(a[2], a[3]));
            if (mx > 0 && mx < GbgcScale<Real>::tiny()) {
                const int sh = -GbgcScale<Real>::expo(mx);     // mx * 2^sh in [1/2, 1)
                const Real f1 = GbgcScale<Real>::pow2(sh / 2), f2 = GbgcScale<Real>::pow2(sh - sh / 2);
#pragma unroll
                for (int j = 0; j < 4; j++) a[j] = (a[j] * f1) * f2;
                e -= sh;
            }
            Real* o = part + ((size_t)s * p.GGp + g) * 4;
#pragma unroll
            for (int j = 0; j < 4; j++) o[j] = a[j];
            p.scl[(size_t)s * p.GGp + g] = e;
        }
        // the root: log sum_j pi_j L_root(j) (log_exp_sum, bpp.hpp:466-474) and its posterior
        Real Lr[4];
        int er;
        gbgc_load(p, p.root, g, Lr, &er);
        double wr[4], tot = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) { wr[j] = (double)Lr[j] * p.pi[j]; tot += wr[j]; }
        if (real_col) p.col[g] = tot > 0 ? log(tot) + (double)er * 0.6931471805599453 : -CUDART_INF;
        // sampling pass (bpp_c.cpp:541-596), top-down; a node's marginal
        // replaces its partial once the node's own terms are formed
        Real* qr = part + ((size_t)p.root * p.GGp + g) * 4;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const double q = (real_col && tot > 0) ? wr[j] / tot : 0.0;
            const double sum = warp_sum(q);
            if (lane == j * 4) wc[p.root * 16 + j * 4] += sum;
            qr[j] = (Real)q;
        }
        for (int k = p.n_nodes - 2; k >= 0; k--) {
            const int s = p.nodes[k];
            if (p.missing[s]) continue;
            Real L[4], m[4];
            int es;
            gbgc_load(p, s, g, L, &es);
            const Real* P = pm + ((size_t)p.cls[s] * p.N + s) * 16;
            gbgc_message(P, L, m);
            const Real* qp = part + ((size_t)p.parent[s] * p.GGp + g) * 4;
            Real r[4];
#pragma unroll
            for (int j = 0; j < 4; j++) r[j] = m[j] > 0 ? qp[j] / m[j] : Real(0);
            Real qs[4];
            double mine = 0;   // lane i*4+j keeps the warp's sum of the (i, j) joint
#pragma unroll
            for (int i = 0; i < 4; i++) {
                Real acc = 0;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const Real jt = r[j] * P[i * 4 + j] * L[i];
                    acc += jt;
                    const double sum = warp_sum(real_col ? (double)jt : 0.0);
                    if (lane == i * 4 + j) mine = sum;
                }
                qs[i] = acc;
            }
            if (lane < 16) wc[s * 16 + lane] += mine;
            if (s >= p.S) {
                Real* o = part + ((size_t)s * p.GGp + g) * 4;
#pragma unroll
                for (int i = 0; i < 4; i++) o[i] = qs[i];
            }
            __syncwarp();
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < p.N * 16; i += blockDim.x) {
        double t = 0;
        for (int v = 0; v < p.warps; v++) t += p.wcounts[(size_t)v * p.N * 16 + i];
        p.counts[i] = t;
    }
}

// prec: 0 FP64 partials, 1 FP32 partials.  p.warps warps in one CTA.
cudaError_t launch_gbgc(const GbgcParams& p, int prec, cudaStream_t st) {
    if (p.n_nodes > 1) {
        const int nt = 6 * (p.n_nodes - 1);
        if (prec == 1) gbgc_pmat_kernel<float><<<(nt + 63) / 64, 64, 0, st>>>(p);
        else gbgc_pmat_kernel<double><<<(nt + 63) / 64, 64, 0, st>>>(p);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (prec == 1) gbgc_engine_kernel<float><<<1, 32 * p.warps, 0, st>>>(p);
    else gbgc_engine_kernel<double><<<1, 32 * p.warps, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace pacc
