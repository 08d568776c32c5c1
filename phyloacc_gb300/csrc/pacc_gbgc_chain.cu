// pacc_gbgc_chain.cu — the PhyloAcc-ST-GBGC chain on the GPU (sm_103a): one
// CTA runs one element through the three models M0, M2, M1 (main.cpp:383-412),
// taking elements from a queue until none are left.
//
// Per iteration the reference (src/PhyloAcc-ST-GBGC/SRC) does
//   MonitorChain (bpp_c.cpp:598-699), the expected-count pass of Update_Tg
//   (bpp_c.cpp:541-596), initial_prob_back (bpp_c2.cpp:354-457), three MH
//   moves of sample_rates with integrate_ZB (bpp_c.cpp:881-976,1765-1799) and
//   update_rates with Update_ZB, a pruning pass and ELBO (bpp_c.cpp:1079-1137,
//   1667-1763, 477-540, 840-878).
// The GPU keeps that sequence and its draw stream, and spreads each step over
// the CTA:
//   * branch matrices: for each class's rate matrix Q = getRate(Q0, s, b) the
//     powers Q^1..Q^13 are formed once (16 threads a class), and each branch's
//     exp(Q d) is the Padé [m/m] approximant of Higham (2005) with m and the
//     scaling chosen from d ||Q||_1, evaluated from the shared powers, in FP64;
//     one thread per (class, branch);
//   * emissions: one thread per (node, class), sum(log P % posterior);
//   * the Z-message pass over log_prob_back: tree levels in parallel, the
//     children of a node added in postorder as the reference adds them (with
//     FP32 partials in FP32 values relative to a per-node FP64 offset);
//   * Z/B sampling: tree depths in parallel, every node's uniform taken at its
//     own position of the stream (one categorical draw per node, in reverse
//     postorder);
//   * pruning and expected counts: one column per lane with linear partials
//     (FP32 or FP64) and exact power-of-two rescaling; counts reduced per warp
//     in a fixed order.
// Partials live in two buffers: the accepted one and the one update_rates
// proposes into; the proposal becomes the accepted one when the move is
// accepted.  Branch matrices of classes 1..5 live in three cache sets: the
// accepted set, the set of the last accepted rate proposal and the set being
// proposed into, so a rejected update_rates restores the caches
// (bpp_c.cpp:318-337) by keeping the old index.
// Eval2 and Output_init run on the host from the traces this kernel writes.
#include "pacc_common.cuh"
#include "pacc_gbgc.cuh"

namespace pacc {

// Padé [m/m] coefficients b_0..b_m of exp for m = 3, 5, 7, 9, 13, and the
// bounds theta_m on ||A||_1 up to which each meets double precision (Higham 2005).
__constant__ double kPadeB[5][14] = {
    {120.0, 60.0, 12.0, 1.0},
    {30240.0, 15120.0, 3360.0, 420.0, 30.0, 1.0},
    {17297280.0, 8648640.0, 1995840.0, 277200.0, 25200.0, 1512.0, 56.0, 1.0},
    {17643225600.0, 8821612800.0, 2075673600.0, 302702400.0, 30270240.0, 2162160.0, 110880.0, 3960.0, 90.0, 1.0},
    {64764752532480000.0, 32382376266240000.0, 7771770303897600.0, 1187353796428800.0, 129060195264000.0,
     10559470521600.0, 670442572800.0, 33522128640.0, 1323241920.0, 40840800.0, 960960.0, 16380.0, 182.0, 1.0}};
__constant__ int kPadeM[5] = {3, 5, 7, 9, 13};
__constant__ double kPadeTheta[5] = {1.495585217958292e-2, 2.539398330063230e-1, 9.504178996162932e-1,
                                     2.097847961257068e0, 5.371920351148152e0};

constexpr int GB_BT = 128;
constexpr int GB_WARPS = GB_BT / 32;
constexpr double LN2 = 0.6931471805599453;

// exp(d Q) from Q's powers pw[k-1] = Q^k (k = 1..13) and ||Q||_1.
// Returns the solve's FP64 flops: 34 m for the sums, 198 for V + U, V - U and
// the 4x4 solve with four right-hand sides, 128 a squaring.
__device__ __noinline__ int pade_branch(const double* __restrict__ pw, double qn, double d, double* E) {
    const double a = qn * d;
    int mi = 0;
    while (mi < 4 && a > kPadeTheta[mi]) mi++;
    int sq = 0;
    if (a > kPadeTheta[4]) sq = (int)ceil(log2(a / kPadeTheta[4]));
    const double sc = ldexp(d, -sq);
    const int m = kPadeM[mi];
    double U[16], V[16];
#pragma unroll
    for (int q = 0; q < 16; q++) { U[q] = 0; V[q] = 0; }
    double c = 1;
    for (int k = 1; k <= m; k++) {
        c *= sc;
        const double bk = kPadeB[mi][k] * c;
        const double* Qk = pw + (k - 1) * 16;
        if (k & 1) {
#pragma unroll
            for (int q = 0; q < 16; q++) U[q] = fma(bk, Qk[q], U[q]);
        } else {
#pragma unroll
            for (int q = 0; q < 16; q++) V[q] = fma(bk, Qk[q], V[q]);
        }
    }
    const double b0 = kPadeB[mi][0];
#pragma unroll
    for (int q = 0; q < 16; q += 5) V[q] += b0;
    // (V - U) E = (V + U): Gaussian elimination with partial pivoting, in
    // place, one reciprocal per pivot
    double rp[4];
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const double u = U[q], v = V[q];
        U[q] = v - u;
        V[q] = v + u;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        int pr = k;
#pragma unroll
        for (int i = k + 1; i < 4; i++)
            if (fabs(U[i * 4 + k]) > fabs(U[pr * 4 + k])) pr = i;
#pragma unroll
        for (int i = k + 1; i < 4; i++)
            if (i == pr)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    double t = U[k * 4 + j]; U[k * 4 + j] = U[i * 4 + j]; U[i * 4 + j] = t;
                    t = V[k * 4 + j]; V[k * 4 + j] = V[i * 4 + j]; V[i * 4 + j] = t;
                }
        rp[k] = 1.0 / U[k * 4 + k];
#pragma unroll
        for (int i = k + 1; i < 4; i++) {
            const double l = U[i * 4 + k] * rp[k];
#pragma unroll
            for (int j = k; j < 4; j++) U[i * 4 + j] -= l * U[k * 4 + j];
#pragma unroll
            for (int j = 0; j < 4; j++) V[i * 4 + j] -= l * V[k * 4 + j];
        }
    }
#pragma unroll
    for (int k = 3; k >= 0; k--)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            double s = V[k * 4 + j];
#pragma unroll
            for (int c2 = k + 1; c2 < 4; c2++) s -= U[k * 4 + c2] * E[c2 * 4 + j];
            E[k * 4 + j] = s * rp[k];
        }
    for (int r = 0; r < sq; r++) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            double row[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                double s = 0;
#pragma unroll
                for (int k = 0; k < 4; k++) s = fma(E[i * 4 + k], E[k * 4 + j], s);
                row[j] = s;
            }
            // rows below i are still read as E's old rows: keep them in V
#pragma unroll
            for (int j = 0; j < 4; j++) V[i * 4 + j] = row[j];
        }
#pragma unroll
        for (int q = 0; q < 16; q++) E[q] = V[q];
    }
    return 34 * m + 198 + 128 * sq;
}

__device__ __forceinline__ unsigned long long gb_timer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ double block_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// log of the Gamma(a, scale b) density (the gsl_ran_gamma_pdf terms of
// sample_rates and MonitorChain, bpp_c.cpp:913-925, 620-642) with lgamma(a)
// and a log(b) computed once: the same terms, in the same order, as
// log_gamma_pdf.
__device__ __noinline__ double lgpdf(double x, double a, double b, double lga, double alb) {
    if (x < 0) return -CUDART_INF;
    if (x == 0) return (a == 1) ? d_log(1.0 / b) : -CUDART_INF;
    const double t = __dsub_rn(__dsub_rn(__dsub_rn(__dmul_rn(a - 1, d_log(x)), __ddiv_rn(x, b)), lga), alb);
    return d_log(d_exp(t));
}

template <typename Real>
__device__ __forceinline__ Real warp_sum_real(Real v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Scalars of one CTA's chain.
struct GbgcScalars {
    double tm[2][3][3], lt[2][3][3];   // Z transition [outgroup path][child Z][parent Z] and its log
    float tmf[2][3][3], ltf[2][3][3];  // the transition and its log in FP32 (the FP32 message pass)
    double ec_gc[2], ec_mis[2];        // emission constants: log(1 - c) / log(c); log(1 - cons2mis) / log(1 - ncons2mis)
    double lmis[4];                    // log(1 - ncons2mis), log(1 - cons2mis), log(ncons2mis), log(cons2mis)
    double pr_lg[3], pr_alb[3];        // lgamma(a) and a log(b) of the conserved, accelerated and GC-bias priors
    int n_all, n_free;                 // branch lists of the model (by length): all, not fixed
    double logpZC, logp_Z, MaxLoglik;
    double tl, tl_next, full;          // trace_loglik[m], trace_loglik[m + 1], trace_full_loglik[m]
    double r_n, r_c, r_gb;             // rates of iteration m
    double x_n, x_c, x_gb;             // the rate proposal
    double lg_x[4];                    // at the chain's (x_gb, x_n, x_c): the three prior terms, log(-x_c)
    double loglik_old, elbo_old, colsum;
    double sel[5], bias[5];
    uint64_t pos;
    int cur, acc, prop, pbuf, post_cur, post_nxt;
    int move_r, changed;
};

template <typename Real>
struct GbgcCtx {
    int S, N, GG, GGp, root, nn, n_int, n_hlev, n_dlev;
    const int16_t *nodes, *c0, *c1, *par, *irank, *pidx, *hlev, *hnodes, *dlev, *dnodes;
    const uint8_t* flags;
    const double* dist;
    const uint8_t* masks;
    double *wc, *emis, *emis_tmp, *lpb, *eraw, *colsum;
    // FP32 partials: log_prob_back as lpo[s] + lpr[s][k] (an FP64 offset a
    // node and six FP32 values), in the memory of lpb
    float* lpr;
    double* lpo;
    Real *lP, *post, *pm, *part;   // log P, expected counts, P, partials in the partials' type
    int32_t* scl;
    Real* Pcur;
    double *pw, *qn;
    int8_t *Z, *B, *fixZ, *Zp, *Bp, *MZ, *MB;
    int16_t *lst_all, *lst_free;   // the model's branches (not missing) by length: all / not fixed
    int nall, nfree;
    __device__ bool missing(int s) const { return flags[s] & GBGC_MISSING; }
    __device__ int upper(int s) const { return (flags[s] & GBGC_UPPER) ? 1 : 0; }
    __device__ int slot(int cls, int set) const { return cls == 0 ? 0 : 1 + 5 * set + (cls - 1); }
    __device__ Real* lp(int sl, int s) const { return lP + ((size_t)sl * N + s) * 16; }
    __device__ Real* pmat(int sl, int s) const { return pm + ((size_t)sl * N + s) * 16; }
    __device__ Real* partial(int buf, int s, int g) const {
        return part + (((size_t)buf * n_int + irank[s]) * GGp + g) * 4;
    }
    __device__ int32_t* expo(int buf, int s, int g) const { return scl + ((size_t)buf * n_int + irank[s]) * GGp + g; }
};

// 16-byte accesses of a 4-vector (a column's partial, a row of P): float4,
// or two double2 (partials and shared rows are 16-byte aligned).
__device__ __forceinline__ void ldv4(const float* p, float* x) {
    const float4 v = *(const float4*)p;
    x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
}
__device__ __forceinline__ void ldv4(const double* p, double* x) {
    const double2 a = ((const double2*)p)[0], b = ((const double2*)p)[1];
    x[0] = a.x; x[1] = a.y; x[2] = b.x; x[3] = b.y;
}
__device__ __forceinline__ void stv4(float* p, const float* x) { *(float4*)p = make_float4(x[0], x[1], x[2], x[3]); }
__device__ __forceinline__ void stv4(double* p, const double* x) {
    ((double2*)p)[0] = make_double2(x[0], x[1]);
    ((double2*)p)[1] = make_double2(x[2], x[3]);
}

// Branch matrices of nc classes (cls[i], selection sel[i], bias bias[i]) into
// cache set `set`; neutral classes are skipped on fixed branches.
template <typename Real>
__device__ void build_caches(const GbgcChainParams& p, const GbgcCtx<Real>& G, int nc, const int* cls,
                             const double* sel, const double* bias, int set) {
    const int tid = threadIdx.x;
    if (tid < nc) {
        double* Q = G.pw + tid * 13 * 16;
        gbgc_rate(p.Q0, sel[tid], bias[tid], Q);
        double n1 = 0;
        for (int j = 0; j < 4; j++) {
            double c = 0;
            for (int i = 0; i < 4; i++) c += fabs(Q[i * 4 + j]);
            n1 = fmax(n1, c);
        }
        G.qn[tid] = n1;
    }
    __syncthreads();
    // powers up to the largest degree any branch of the list needs (the
    // longest branch of the element is the last of the list; scaling and
    // squaring only with degree 13)
    int kmax = 3;
    {
        const double dmax = G.nall > 0 ? G.dist[G.lst_all[G.nall - 1]] : 0.0;
        for (int i = 0; i < nc; i++) {
            const double a = G.qn[i] * dmax;
            int mi = 0;
            while (mi < 4 && a > kPadeTheta[mi]) mi++;
            kmax = max(kmax, kPadeM[mi]);
        }
    }
    for (int k = 2; k <= kmax; k++) {
        if (tid < nc * 16) {
            const int ci = tid >> 4, e = tid & 15, r = e >> 2, c = e & 3;
            double* Qm = G.pw + ci * 13 * 16;
            const double* Qp = Qm + (k - 2) * 16;
            double s = 0;
            for (int l = 0; l < 4; l++) s = fma(Qp[r * 4 + l], Qm[l * 4 + c], s);
            Qm[(k - 1) * 16 + e] = s;   // writes row k-1 only; rows read are k-2 and 0
        }
        __syncthreads();
    }
    // work items: each class over its branch list (the neutral classes skip
    // fixed branches), branches by length so a warp's lanes choose the same
    // Padé degree
    int cnt[5], tot = 0;
    for (int i = 0; i < nc; i++) {
        cnt[i] = (cls[i] % 3 == 2) ? G.nfree : G.nall;
        tot += cnt[i];
    }
    unsigned fl = 0;
    for (int it = tid; it < tot; it += blockDim.x) {
        int ci = 0, k = it;
        while (k >= cnt[ci]) { k -= cnt[ci]; ci++; }
        const int s = (cls[ci] % 3 == 2) ? G.lst_free[k] : G.lst_all[k];
        double E[16];
        fl += (unsigned)pade_branch(G.pw + ci * 13 * 16, G.qn[ci], G.dist[s], E);
        const int sl = G.slot(cls[ci], set);
        Real* lo = G.lp(sl, s);
        Real* po = G.pmat(sl, s);
        if constexpr (sizeof(Real) == 4) {
            // FP32 partials: log P in FP32 (an error below the one the
            // partials put on the expected counts it multiplies), one
            // conversion an entry; the diagonal (close to 1 on short
            // branches) as log1p of minus its row's off-diagonal sum (rows of
            // exp(dQ) sum to one)
            float ef[16];
#pragma unroll
            for (int q = 0; q < 16; q++) ef[q] = (float)E[q];
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const int r = q & 3, c = q >> 2;   // (child c, parent r) = E[r][c]
                const float v = ef[r * 4 + c];
                float l;
                if (r == c) {
                    float off = 0;
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if (j != r) off += ef[r * 4 + j];
                    l = log1pf(-off);
                } else {
                    l = logf(v);
                }
                lo[q] = l;
                po[q] = v;
            }
        } else {
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const double v = E[(q & 3) * 4 + (q >> 2)];   // (child q/4, parent q%4) = E[parent][child]
                lo[q] = d_log(v);
                po[q] = (Real)v;
            }
        }
    }
    if (p.flop) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) fl += __shfl_xor_sync(0xffffffffu, fl, o);
        if ((tid & 31) == 0) atomicAdd(p.flop, (unsigned long long)fl);
    }
    __syncthreads();
}

// Emissions sum(log P % posterior) (+ the B and missing-data constants) of the
// classes lo..5 from cache set `set` into out; with raw, the value of each
// node's current class before the constants goes to eraw.
template <typename Real>
__device__ void emissions(const GbgcCtx<Real>& G, const GbgcScalars& sc, double* out, int lo, int set,
                          const Real* post, bool raw) {
    const int nb = G.nn - 1, ncl = 6 - lo;
    for (int it = threadIdx.x; it < nb * ncl; it += blockDim.x) {
        const int s = G.nodes[it / ncl], j = lo + it % ncl;
        if (G.missing(s) || (G.fixZ[s] == 1 && j % 3 == 2)) continue;
        Real a[16], b[16];
#pragma unroll
        for (int q = 0; q < 16; q += 4) {
            ldv4(G.lp(G.slot(j, set), s) + q, a + q);
            ldv4(post + (size_t)s * 16 + q, b + q);
        }
        Real tr = 0;
#pragma unroll
        for (int c = 0; c < 4; c++)
#pragma unroll
            for (int r = 0; r < 4; r++) tr += a[r * 4 + c] * b[r * 4 + c];
        double t = (double)tr;
        if (raw && j == G.Z[s] + 3 * G.B[s]) G.eraw[s] = t;
        t += sc.ec_gc[j < 3 ? 0 : 1];
        t += sc.ec_mis[j % 3 == 1 ? 0 : 1];
        out[s * 6 + j] = t;
    }
    __syncthreads();
}

// log_multi of the 6 x 3 log_TM_Int by log_prob_back y (max mx), in linear
// space: t_j = mx + log(sum_z TM[z][j] (e^(y_z - mx) + e^(y_(z+3) - mx))), in
// FP64 (the FP64-partial path; the FP32 path's message pass has its own form).
__device__ __forceinline__ void lm63(const GbgcScalars& sc, int u, const double* y, double mx, double* t) {
    const double (*tm)[3] = sc.tm[u];
    double ez[3];
#pragma unroll
    for (int z = 0; z < 3; z++) ez[z] = d_exp(y[z] - mx) + d_exp(y[z + 3] - mx);
#pragma unroll
    for (int j = 0; j < 3; j++) {
        double v = 0;
#pragma unroll
        for (int z = 0; z < 3; z++) v += tm[z][j] * ez[z];
        t[j] = d_log(v) + mx;
    }
}

// The Z-message pass: lpb[p] += log_multi(log_TM_Int[c], lpb[c]) (- log 2)
// for every non-root c, bottom-up.
template <typename Real>
__device__ void up_pass(const GbgcCtx<Real>& G, const GbgcScalars& sc, bool half) {
    if constexpr (sizeof(Real) == 4) {
        // FP32 partials: the values relative to each node's FP64 offset in
        // FP32; a child's maximum goes to the parent's offset, so FP64 work
        // is two additions a child (the FP64 pipe is narrow and these
        // levels run on few threads)
        for (int h = 0; h < G.n_hlev; h++) {
            const int a = G.hlev[h], b = G.hlev[h + 1];
            for (int it = a + threadIdx.x; it < b; it += blockDim.x) {
                const int p = G.hnodes[it];
                float acc[6];
#pragma unroll
                for (int r = 0; r < 6; r++) acc[r] = G.lpr[p * 6 + r];
                double off = G.lpo[p];
                const int ch[2] = {G.c0[p], G.c1[p]};
                for (int q = 0; q < 2; q++) {
                    const int c = ch[q];
                    const float* y = G.lpr + c * 6;
                    float mx = y[0];
#pragma unroll
                    for (int r = 1; r < 6; r++) mx = fmaxf(mx, y[r]);
                    float t[3];
                    if (mx == -CUDART_INF_F) {
                        t[0] = t[1] = t[2] = -CUDART_INF_F;
                    } else {
                        const float (*tm)[3] = sc.tmf[G.upper(c)];
                        float ez[3];
#pragma unroll
                        for (int z = 0; z < 3; z++) ez[z] = expf(y[z] - mx) + expf(y[z + 3] - mx);
#pragma unroll
                        for (int j = 0; j < 3; j++) {
                            float v = 0;
#pragma unroll
                            for (int z = 0; z < 3; z++) v += tm[z][j] * ez[z];
                            t[j] = logf(v) - (half ? (float)LN2 : 0.0f);
                        }
                        off += G.lpo[c] + (double)mx;
                    }
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        acc[j] += t[j];
                        acc[3 + j] += t[j];
                    }
                }
#pragma unroll
                for (int r = 0; r < 6; r++) G.lpr[p * 6 + r] = acc[r];
                G.lpo[p] = off;
            }
            __syncthreads();
        }
    } else {
        for (int h = 0; h < G.n_hlev; h++) {
            const int a = G.hlev[h], b = G.hlev[h + 1];
            for (int it = a + threadIdx.x; it < b; it += blockDim.x) {
                const int p = G.hnodes[it];
                double acc[6];
#pragma unroll
                for (int r = 0; r < 6; r++) acc[r] = G.lpb[p * 6 + r];
                const int ch[2] = {G.c0[p], G.c1[p]};
                for (int q = 0; q < 2; q++) {
                    const int c = ch[q];
                    const double* y = G.lpb + c * 6;
                    double mx = y[0];
#pragma unroll
                    for (int r = 1; r < 6; r++) mx = fmax(mx, y[r]);
                    double t[3];
                    if (mx == -CUDART_INF) {
                        t[0] = t[1] = t[2] = -CUDART_INF;
                    } else {
                        lm63(sc, G.upper(c), y, mx, t);
#pragma unroll
                        for (int j = 0; j < 3; j++)
                            if (half) t[j] -= LN2;
                    }
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        acc[j] += t[j];
                        acc[3 + j] += t[j];
                    }
                }
#pragma unroll
                for (int r = 0; r < 6; r++) G.lpb[p * 6 + r] = acc[r];
            }
            __syncthreads();
        }
    }
}

// log_prob_back of the root's first class (the integrated log-likelihood).
template <typename Real>
__device__ __forceinline__ double lpb_root(const GbgcCtx<Real>& G) {
    if constexpr (sizeof(Real) == 4) return G.lpo[G.root] + (double)G.lpr[G.root * 6];
    else return G.lpb[G.root * 6];
}

// lpb = src on the branches, 0 at the root, then the message pass.
template <typename Real>
__device__ void prob_back(const GbgcCtx<Real>& G, const GbgcScalars& sc, const double* src) {
    if constexpr (sizeof(Real) == 4) {
        // offset: the node's largest finite value
        for (int k = threadIdx.x; k < G.nn; k += blockDim.x) {
            const int s = G.nodes[k];
            if (s == G.root) {
                G.lpo[s] = 0;
#pragma unroll
                for (int r = 0; r < 6; r++) G.lpr[s * 6 + r] = 0.0f;
                continue;
            }
            double v[6], m = -CUDART_INF;
#pragma unroll
            for (int r = 0; r < 6; r++) {
                v[r] = src[s * 6 + r];
                if (v[r] > m && v[r] < CUDART_INF) m = v[r];
            }
            if (m == -CUDART_INF) m = 0;
            G.lpo[s] = m;
#pragma unroll
            for (int r = 0; r < 6; r++) G.lpr[s * 6 + r] = (float)(v[r] - m);
        }
        __syncthreads();
        up_pass(G, sc, false);
    } else {
        for (int i = threadIdx.x; i < G.nn * 6; i += blockDim.x) {
            const int s = G.nodes[i / 6];
            G.lpb[s * 6 + i % 6] = (s == G.root) ? 0.0 : src[s * 6 + i % 6];
        }
        __syncthreads();
        up_pass(G, sc, false);
    }
}

// The current class's matrices of every branch into shared memory.
template <typename Real>
__device__ void stage_pcur(const GbgcCtx<Real>& G, int set) {
    for (int i = threadIdx.x; i < (G.nn - 1) * 16; i += blockDim.x) {
        const int s = G.nodes[i >> 4];
        const int k = G.Z[s] + 3 * G.B[s];
        G.Pcur[s * 16 + (i & 15)] = (G.missing(s) || k < 0) ? Real(0) : G.pmat(G.slot(k, set), s)[i & 15];
    }
    __syncthreads();
}

// log(sum_j pi_j L_root(j)) + e log 2 of one column: FP64 with FP64
// partials; with FP32 partials the sum and its logarithm in FP32 (the
// partials' own error is larger), the exponent term in FP64.
__device__ __forceinline__ double column_loglik(const double* L, const double* pi, int e) {
    double t = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) t += L[j] * pi[j];
    return t > 0 ? d_log(t) + (double)e * LN2 : -CUDART_INF;
}
__device__ __forceinline__ double column_loglik(const float* L, const double* pi, int e) {
    float t = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) t += L[j] * (float)pi[j];
    return t > 0 ? (double)logf(t) + (double)e * LN2 : -CUDART_INF;
}

// gbgc_message with P's rows read as 4-vectors (the same arithmetic).
template <typename Real>
__device__ __forceinline__ void message_v(const Real* P, const Real* L, Real* m) {
    Real r0[4], r1[4], r2[4], r3[4];
    ldv4(P, r0); ldv4(P + 4, r1); ldv4(P + 8, r2); ldv4(P + 12, r3);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        Real v = r0[j] * L[0];
        v = fma(r1[j], L[1], v);
        v = fma(r2[j], L[2], v);
        v = fma(r3[j], L[3], v);
        m[j] = v;
    }
}

template <typename Real>
__device__ __forceinline__ void leaf_or_partial(const GbgcCtx<Real>& G, int buf, int s, int g, Real* L, int* e) {
    if (s < G.S) {
        const int msk = G.masks[(size_t)s * G.GGp + g];
#pragma unroll
        for (int i = 0; i < 4; i++) L[i] = ((msk >> i) & 1) ? Real(1) : Real(0);
        *e = 0;
    } else {
        ldv4(G.partial(buf, s, g), L);
        *e = *G.expo(buf, s, g);
    }
}

// Update_Tg without sampling over every column into partial buffer buf;
// returns (in sc.colsum) sum over columns of log(sum_j pi_j L_root(j)).
template <typename Real>
__device__ void prune(const GbgcChainParams& p, const GbgcCtx<Real>& G, GbgcScalars& sc, int buf) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double tot = 0;
    for (int g0 = w * 32; g0 < G.GGp; g0 += GB_WARPS * 32) {
        const int g = g0 + lane;
        for (int k = 0; k < G.nn; k++) {
            const int s = G.nodes[k];
            if (s < G.S || G.missing(s)) continue;
            Real a[4] = {1, 1, 1, 1};
            int e = 0;
            const int ch[2] = {G.c0[s], G.c1[s]};
            for (int q = 0; q < 2; q++) {
                const int c = ch[q];
                if (G.missing(c)) continue;
                Real L[4], m[4];
                int ec;
                leaf_or_partial(G, buf, c, g, L, &ec);
                message_v(G.Pcur + c * 16, L, m);
#pragma unroll
                for (int j = 0; j < 4; j++) a[j] *= m[j];
                e += ec;
            }
            const Real mx = fmax(fmax(a[0], a[1]), fmax(a[2], a[3]));
            if (mx > 0 && mx < GbgcScale<Real>::tiny()) {
                const int sh = -GbgcScale<Real>::expo(mx);
                const Real f1 = GbgcScale<Real>::pow2(sh / 2), f2 = GbgcScale<Real>::pow2(sh - sh / 2);
#pragma unroll
                for (int j = 0; j < 4; j++) a[j] = (a[j] * f1) * f2;
                e -= sh;
            }
            stv4(G.partial(buf, s, g), a);
            *G.expo(buf, s, g) = e;
        }
        if (g < G.GG) {
            Real Lr[4];
            int er;
            leaf_or_partial(G, buf, G.root, g, Lr, &er);
            tot += column_loglik(Lr, p.pi, er);
        }
    }
    tot = block_warp_sum(tot);
    if (lane == 0) G.colsum[w] = tot;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int v = 0; v < GB_WARPS; v++) t += G.colsum[v];
        sc.colsum = t;
    }
    __syncthreads();
}

// q / m in the expected-count pass: exact in FP64; with FP32 partials the
// fast FP32 quotient (within 2 ulp), far inside the partials' own error.
__device__ __forceinline__ double gb_div(double q, double m) { return q / m; }
__device__ __forceinline__ float gb_div(float q, float m) { return __fdividef(q, m); }

// Reduce-scatter of 16 values across a warp by recursive halving (16
// shuffles): afterwards lane l holds the warp's sum of value (l >> 1) & 15
// (lanes 2i and 2i + 1 both hold sum i).  The order of the additions depends
// only on the lane numbers.
template <typename Real>
__device__ __forceinline__ Real warp_reduce_scatter16(Real* v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 16, h = 8; o >= 2; o >>= 1, h >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < h; i++) {
            const Real send = up ? v[i] : v[i + h];
            const Real keep = up ? v[i + h] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

// Update_Tg with sampling over every column from partial buffer buf (its
// internal partials are replaced by marginals): expected counts into dst.
// Nodes top-down in the outer loop and a thread's columns in the inner one:
// a node's joint counts are summed over the thread's columns in registers,
// then once over the warp (reduce-scatter) into the warp's slice, and the
// slices are summed in warp order.  Column g stays on thread g mod blockDim,
// so the parent's marginal a thread reads is one it wrote itself.
template <typename Real>
__device__ void counts(const GbgcChainParams& p, const GbgcCtx<Real>& G, int buf, Real* dst) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // per-warp sums in the partials' type (FP32 sums stay off the FP64 pipe)
    Real* wc = (Real*)G.wc + (size_t)w * G.N * 16;
    for (int i = lane; i < G.N * 16; i += 32) wc[i] = 0;
    __syncwarp();
    {
        // the root: posterior of each column (root marginal stored in place)
        Real acc[16];
#pragma unroll
        for (int q = 0; q < 16; q++) acc[q] = 0;
        for (int g = threadIdx.x; g < G.GG; g += blockDim.x) {
            Real Lr[4];
            int er;
            leaf_or_partial(G, buf, G.root, g, Lr, &er);
            Real wr[4], tot = 0;
#pragma unroll
            for (int j = 0; j < 4; j++) { wr[j] = Lr[j] * (Real)p.pi[j]; tot += wr[j]; }
            Real qv[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                qv[j] = tot > 0 ? gb_div(wr[j], tot) : Real(0);
                acc[j * 4] += qv[j];
            }
            stv4(G.partial(buf, G.root, g), qv);
        }
        const Real sum = warp_reduce_scatter16(acc);
        if ((lane & 1) == 0) wc[G.root * 16 + (lane >> 1)] = sum;
    }
    for (int k = G.nn - 2; k >= 0; k--) {
        const int s = G.nodes[k];
        if (G.missing(s)) continue;
        const Real* P = G.Pcur + s * 16;
        Real acc[16];
#pragma unroll
        for (int q = 0; q < 16; q++) acc[q] = 0;
        for (int g = threadIdx.x; g < G.GG; g += blockDim.x) {
            Real L[4], m[4];
            int es;
            leaf_or_partial(G, buf, s, g, L, &es);
            // P's rows once for the message and the joint terms
            Real pr[4][4];
            ldv4(P, pr[0]); ldv4(P + 4, pr[1]); ldv4(P + 8, pr[2]); ldv4(P + 12, pr[3]);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                Real v = pr[0][j] * L[0];
                v = fma(pr[1][j], L[1], v);
                v = fma(pr[2][j], L[2], v);
                v = fma(pr[3][j], L[3], v);
                m[j] = v;
            }
            Real qp[4];
            ldv4(G.partial(buf, G.par[s], g), qp);
            Real r[4];
#pragma unroll
            for (int j = 0; j < 4; j++) r[j] = m[j] > 0 ? gb_div(qp[j], m[j]) : Real(0);
            Real qs[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                Real a = 0;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const Real jt = r[j] * pr[i][j] * L[i];
                    a += jt;
                    acc[i * 4 + j] += jt;
                }
                qs[i] = a;
            }
            if (s >= G.S) stv4(G.partial(buf, s, g), qs);
        }
        const Real sum = warp_reduce_scatter16(acc);
        if ((lane & 1) == 0) wc[s * 16 + (lane >> 1)] = sum;
    }
    __syncthreads();
    const Real* wa = (const Real*)G.wc;
    for (int i = threadIdx.x; i < G.N * 16; i += blockDim.x) {
        Real t = 0;
        for (int v = 0; v < GB_WARPS; v++) t += wa[(size_t)v * G.N * 16 + i];
        dst[i] = t;
    }
    __syncthreads();
}

// Inverse-CDF draw over K unnormalised FP32 weights with the 24-bit uniform
// ((w >> 8) + 0.5) 2^-24 of word w: the first k with u * total below the
// k-th cumulative sum.
__device__ __forceinline__ int categorical_f(int K, const float* p, uint32_t w) {
    const float u = ((float)(w >> 8) + 0.5f) * 5.9604644775390625e-08f;
    float tot = 0;
    for (int k = 0; k < K; k++) tot += p[k];
    const float t = u * tot;
    float cum = 0;
    for (int k = 0; k < K; k++) {
        cum += p[k];
        if (t < cum) return k;
    }
    for (int k = K - 1; k >= 0; k--)
        if (p[k] > 0) return k;
    return K;
}

// Update_ZB's sampling (bpp_c.cpp:1710-1761): depths top-down, the node at
// reverse-postorder index k drawing the uniform at position pos0 + k.
template <typename Real>
__device__ void sample_zb(const GbgcChainParams& p, const GbgcCtx<Real>& G, GbgcScalars& sc) {
    for (int d = 0; d < G.n_dlev; d++) {
        const int a = G.dlev[d], b = G.dlev[d + 1];
        for (int it = a + threadIdx.x; it < b; it += blockDim.x) {
            const int s = G.dnodes[it], pz = G.Z[G.par[s]];
            StreamReader rd;
            rd.init(p.seed, sc.pos + (uint64_t)(G.nn - 2 - G.pidx[s]));
            const int old = G.Z[s];
            if constexpr (sizeof(Real) == 4) {
                // FP32 weights from the FP32 values (the node's offset cancels)
                // and the word's 24-bit uniform
                const uint32_t wd = rd.word_at(rd.pos);
                const float* y = G.lpr + s * 6;
                if (pz != 2) {
                    float x[6], wv[6];
                    const int up = G.upper(s);
#pragma unroll
                    for (int r = 0; r < 6; r++) x[r] = sc.ltf[up][r % 3][pz] + y[r];
                    float mx = x[0];
#pragma unroll
                    for (int r = 1; r < 6; r++) mx = fmaxf(mx, x[r]);
#pragma unroll
                    for (int r = 0; r < 6; r++) wv[r] = expf(x[r] - mx);
                    const int nn = categorical_f(6, wv, wd);
                    G.Z[s] = (int8_t)(nn % 3);
                    if (!G.missing(s)) G.B[s] = nn > 2 ? 1 : 0;
                } else {
                    G.Z[s] = 2;
                    const float mx = fmaxf(y[2], y[5]);
                    const float wv[2] = {expf(y[2] - mx), expf(y[5] - mx)};
                    const int nn = categorical_f(2, wv, wd);
                    if (!G.missing(s)) G.B[s] = nn > 0 ? 1 : 0;
                }
                if (old != G.Z[s]) sc.changed = 1;
            } else {
                const double u = rd.uniform();
                const double* y = G.lpb + s * 6;
                if (pz != 2) {
                    double x[6], wv[6];
                    const int up = G.upper(s);
#pragma unroll
                    for (int r = 0; r < 6; r++) x[r] = sc.lt[up][r % 3][pz] + y[r];
                    double mx = x[0];
#pragma unroll
                    for (int r = 1; r < 6; r++)
                        if (x[r] > mx) mx = x[r];
#pragma unroll
                    for (int r = 0; r < 6; r++) wv[r] = d_exp(x[r] - mx);
                    const int nn = categorical(6, wv, u);
                    G.Z[s] = (int8_t)(nn % 3);
                    if (!G.missing(s)) G.B[s] = nn > 2 ? 1 : 0;
                } else {
                    G.Z[s] = 2;
                    const double mx = fmax(y[2], y[5]);
                    const double wv[2] = {d_exp(y[2] - mx), d_exp(y[5] - mx)};
                    const int nn = categorical(2, wv, u);
                    if (!G.missing(s)) G.B[s] = nn > 0 ? 1 : 0;
                }
                if (old != G.Z[s]) sc.changed = 1;
            }
        }
        __syncthreads();
    }
}

// prior_Z (bpp_c2.cpp:484-498), reverse postorder
template <typename Real>
__device__ double prior_z(const GbgcCtx<Real>& G, const GbgcScalars& sc) {
    double r = 0;
    for (int k = G.nn - 2; k >= 0; k--) {
        const int s = G.nodes[k];
        r += sc.lt[G.upper(s)][G.Z[s]][G.Z[G.par[s]]];
    }
    return r;
}

template <typename Real, int MINB>
__global__ void __launch_bounds__(GB_BT, MINB) gbgc_chain_kernel(GbgcChainParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ GbgcScalars sc;
    __shared__ int s_elem;
    // phase clock (thread 0, at phase ends that follow a block barrier):
    // 0 monitor and init, 1 expected counts, 2 initial_prob_back, 3 branch
    // matrices of the rate proposals, 4 the rest of sample_rates, 5 Update_ZB,
    // 6 pruning, 7 ELBO and update_rates' MH
    __shared__ unsigned long long s_ph[8];
    __shared__ long long s_t;
#define GB_MARK(i)                                          \
    if (p.phase && tid == 0) {                              \
        const long long t_ = clock64();                     \
        s_ph[i] += (unsigned long long)(t_ - s_t);          \
        s_t = t_;                                           \
    }
    const int tid = threadIdx.x;
    StreamReader rng;   // thread 0's sequential reader
    for (;;) {
        if (tid == 0) {
            if (!p.stream) {
                s_elem = atomicAdd(p.next_elem, 1);
            } else {
                // the next published queue position; return when the host asks
                // idle blocks to stop, or after idle_ns without work
                s_elem = p.n_elem;
                const unsigned long long t0 = gb_timer_ns();
                for (;;) {
                    const int h = *(volatile int*)p.q_head;
                    const int t = *p.q_tail;
                    if (h >= t && *p.q_stop) break;
                    if (h < t) {
                        if (atomicCAS(p.q_head, h, h + 1) == h) {
                            __threadfence_system();   // the slot id and its data after the tail
                            s_elem = p.q_slot[h % p.q_cap];
                            break;
                        }
                        continue;
                    }
                    if ((long long)(gb_timer_ns() - t0) > p.idle_ns) {
                        if (p.idle_exits) atomicAdd(p.idle_exits, 1ull);
                        break;
                    }
                    __nanosleep(4000);
                }
            }
        }
        __syncthreads();
        const int e = s_elem;
        if (e < 0 || e >= p.n_elem) break;
        GbgcElemHdr H;
        if (p.stream) {
            // the host rewrote this slot while the kernel ran: read it past L1
            const int* src = (const int*)(p.hdr + e);
            int* dst = (int*)&H;
            for (int i = 0; i < (int)(sizeof(GbgcElemHdr) / 4); i++) dst[i] = __ldcg(src + i);
        } else {
            H = p.hdr[e];
        }
        const uint8_t* eb = p.blob + H.blob_off;
        GbgcCtx<Real> G;
        G.S = H.S; G.N = H.N; G.GG = H.GG; G.GGp = H.GGp; G.root = H.root; G.nn = H.n_nodes; G.n_int = H.n_int;
        G.n_hlev = H.n_hlev; G.n_dlev = H.n_dlev;
        const int N = G.N;
        // shared layout
        size_t o = 0;
        G.Pcur = (Real*)(smem + o);   o += (size_t)N * 16 * sizeof(Real);
        G.pw = (double*)(smem + o);   o += 5 * 13 * 16 * 8;
        G.qn = (double*)(smem + o);   o += 8 * 8;
        int16_t* i16 = (int16_t*)(smem + o);
        const int nh = H.n_hlev + 1, nd = H.n_dlev + 1, nhn = H.n_int, ndn = G.nn - 1;
        o += ((size_t)6 * N + nh + nhn + nd + ndn) * 2;
        G.lst_all = (int16_t*)(smem + o);
        G.lst_free = G.lst_all + N;
        o += (size_t)4 * N;
        o = (o + 15) & ~(size_t)15;
        uint8_t* u8 = smem + o;
        for (int i = tid; i < N; i += blockDim.x) {
            i16[i] = i < G.nn ? ((const int16_t*)(eb + H.o_nodes))[i] : 0;
            i16[N + i] = ((const int16_t*)(eb + H.o_c0))[i];
            i16[2 * N + i] = ((const int16_t*)(eb + H.o_c1))[i];
            i16[3 * N + i] = ((const int16_t*)(eb + H.o_par))[i];
            i16[4 * N + i] = ((const int16_t*)(eb + H.o_irank))[i];
            i16[5 * N + i] = ((const int16_t*)(eb + H.o_pidx))[i];
            u8[i] = (eb + H.o_flags)[i] | (p.target[i] ? GBGC_TARGET : 0);
        }
        int16_t* lv = i16 + 6 * N;
        for (int i = tid; i < nh; i += blockDim.x) lv[i] = ((const int16_t*)(eb + H.o_hlev))[i];
        for (int i = tid; i < nhn; i += blockDim.x) lv[nh + i] = ((const int16_t*)(eb + H.o_hnodes))[i];
        for (int i = tid; i < nd; i += blockDim.x) lv[nh + nhn + i] = ((const int16_t*)(eb + H.o_dlev))[i];
        for (int i = tid; i < ndn; i += blockDim.x) lv[nh + nhn + nd + i] = ((const int16_t*)(eb + H.o_dnodes))[i];
        for (int i = tid; i < H.n_blen; i += blockDim.x) G.lst_all[i] = ((const int16_t*)(eb + H.o_blen))[i];
        G.nall = H.n_blen;
        G.nodes = i16; G.c0 = i16 + N; G.c1 = i16 + 2 * N; G.par = i16 + 3 * N; G.irank = i16 + 4 * N;
        G.pidx = i16 + 5 * N;
        G.hlev = lv; G.hnodes = lv + nh; G.dlev = lv + nh + nhn; G.dnodes = lv + nh + nhn + nd;
        G.flags = u8;
        G.Z = (int8_t*)u8 + N; G.B = G.Z + N; G.fixZ = G.B + N; G.Zp = G.fixZ + N; G.Bp = G.Zp + N;
        G.MZ = G.Bp + N; G.MB = G.MZ + N;
        G.dist = (const double*)(eb + H.o_dist);
        G.masks = eb + H.o_masks;
        const GbgcWs W = GbgcWs::make(p.N_max, p.n_int_max, p.GGp_max, GB_WARPS, sizeof(Real));
        char* ws = p.ws + (size_t)blockIdx.x * p.ws_stride;
        G.lP = (Real*)(ws + W.lP); G.pm = (Real*)(ws + W.pm); G.post = (Real*)(ws + W.post);
        G.wc = (double*)(ws + W.wc); G.emis = (double*)(ws + W.emis); G.emis_tmp = (double*)(ws + W.emis_tmp);
        G.lpb = (double*)(ws + W.lpb); G.eraw = (double*)(ws + W.eraw); G.colsum = (double*)(ws + W.colsum);
        G.lpr = (float*)G.lpb;
        G.lpo = (double*)(G.lpr + (size_t)N * 6);   // 24 N + 8 N bytes within lpb's 48 N
        G.part = (Real*)(ws + W.part); G.scl = (int32_t*)(ws + W.scl);
        if (tid == 0) {
            for (int q = 0; q < 8; q++) s_ph[q] = 0;
            s_t = clock64();
            for (int u = 0; u < 2; u++) {
                double t[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                t[0][0] = 1 - p.grate;
                t[1][0] = p.grate;
                t[1][1] = 1 - p.lrate;
                t[2][1] = p.lrate;
                t[2][2] = 1;
                if (u) { t[1][1] = 1; t[2][1] = 0; }
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) {
                        sc.tm[u][a][b] = t[a][b];
                        sc.tmf[u][a][b] = (float)t[a][b];
                        sc.lt[u][a][b] = d_log(t[a][b]);
                        sc.ltf[u][a][b] = (float)sc.lt[u][a][b];
                    }
            }
            sc.ec_gc[0] = d_log(1 - p.gcc);
            sc.ec_gc[1] = d_log(p.gcc);
            sc.ec_mis[0] = d_log(1 - p.c2m);
            sc.ec_mis[1] = d_log(1 - p.nc2m);
            sc.lmis[0] = d_log(1 - p.nc2m);
            sc.lmis[1] = d_log(1 - p.c2m);
            sc.lmis[2] = d_log(p.nc2m);
            sc.lmis[3] = d_log(p.c2m);
            const double pa[3] = {p.ca, p.na, p.gca}, pb[3] = {p.cb, p.nb, p.gcb};
            for (int q = 0; q < 3; q++) {
                sc.pr_lg[q] = d_lgamma(pa[q]);
                sc.pr_alb[q] = __dmul_rn(pa[q], d_log(pb[q]));
            }
            rng.init(p.seed, 0);
        }
        __syncthreads();
        const int order[3] = {0, 2, 1};
        for (int q = 0; q < 3; q++) {
            const int resZ = order[q];
            double* trd = p.tr_d + ((size_t)e * 3 + resZ) * 4 * p.T;
            int8_t* trzb = p.tr_zb + ((size_t)e * 3 + resZ) * p.T * 2 * p.N_max;
            // ---- initMCMC (bpp_c.cpp:120-257) ----
            for (int s = tid; s < N; s += blockDim.x) {
                G.B[s] = 0;
                G.Z[s] = p.chain > 0 ? 0 : -1;   // a later chain: bpp.cur_Z, all zeros
                int f = -1;
                if (G.upper(s)) f = 1;
                if (resZ == 2 && s < G.S) f = (G.flags[s] & GBGC_TARGET) ? -1 : 1;
                G.fixZ[s] = (int8_t)f;
                G.MZ[s] = 0;
                G.MB[s] = 0;
            }
            __syncthreads();
            for (int k = tid; k < G.nn; k += blockDim.x) {
                const int s = G.nodes[k];
                G.Z[s] = 0;
                int f = G.upper(s) ? 1 : -1;
                if (resZ == 2 && s < G.S) f = (G.flags[s] & GBGC_TARGET) ? -1 : 1;
                if (resZ == 0) f = 1;
                if (s == G.root) f = 0;
                G.fixZ[s] = (int8_t)f;
            }
            __syncthreads();
            if (tid == 0) {
                int k = 0;
                for (int i = 0; i < G.nall; i++)
                    if (G.fixZ[G.lst_all[i]] != 1) G.lst_free[k++] = G.lst_all[i];
                sc.n_free = k;
            }
            __syncthreads();
            G.nfree = sc.n_free;
            if (tid == 0) {
                sc.MaxLoglik = -CUDART_INF;
                sc.r_n = p.acce_rate;
                sc.r_c = p.conserve_rate;
                sc.r_gb = p.init_gc;
                sc.cur = 0;
                sc.pbuf = 0;
                sc.post_cur = 0;
                sc.post_nxt = 0;
            }
            __syncthreads();
            {
                const int cls[5] = {1, 2, 3, 4, 5};
                const double sel[5] = {sc.r_c, sc.r_n, 0.0, sc.r_c, sc.r_n};
                const double bias[5] = {0.0, 0.0, sc.r_gb, sc.r_gb, sc.r_gb};
                const int c0[1] = {0};
                const double z0[1] = {0.0};
                build_caches(p, G, 1, c0, z0, z0, 0);
                build_caches(p, G, 5, cls, sel, bias, 0);
            }
            const double lnc = d_log(p.nc2m), lc = d_log(p.c2m);
            for (int i = tid; i < N * 6; i += blockDim.x) {
                const int s = i / 6, j = i % 6;
                const bool ban = G.fixZ[s] == 1 && j % 3 == 2;
                if constexpr (sizeof(Real) == 4) {
                    G.lpr[i] = ban ? -CUDART_INF_F : 0.0f;
                    if (j == 0) G.lpo[s] = 0;
                } else {
                    G.lpb[i] = ban ? -CUDART_INF : 0.0;
                }
                G.emis[i] = ban ? -CUDART_INF : 0.0;
            }
            __syncthreads();
            for (int k = tid; k < G.nn - 1; k += blockDim.x) {
                const int s = G.nodes[k];
                if (G.missing(G.par[s]) || !G.missing(s)) continue;
                for (int j = 0; j < 6; j++) {
                    if (G.fixZ[s] == 1 && j % 3 == 2) continue;
                    G.emis[s * 6 + j] = (j % 3 == 1) ? lc : lnc;
                }
            }
            __syncthreads();
            up_pass(G, sc, true);
            if (tid == 0) sc.logpZC = lpb_root(G);
            __syncthreads();
            // ---- Gibbs (bpp_c.cpp:259-349) ----
            stage_pcur(G, sc.cur);
            prune(p, G, sc, sc.pbuf);
            if (tid == 0) {
                sc.tl = sc.colsum;
                sc.logp_Z = prior_z(G, sc) - sc.logpZC;
                sc.move_r = 1;
            }
            __syncthreads();
            for (int m = 0; m < p.T; m++) {
                // MonitorChain
                if (tid == 0) {
                    if (m > 0) {
                        if (sc.move_r) sc.tl = sc.tl_next;
                    }
                    if (sc.move_r) {
                        double f = sc.tl + sc.logp_Z;
                        f += lgpdf(-sc.r_c, p.ca, p.cb, sc.pr_lg[0], sc.pr_alb[0]);
                        if (resZ != 0) f += lgpdf(sc.r_n + p.nshift, p.na, p.nb, sc.pr_lg[1], sc.pr_alb[1]);
                        int gb = 0, ungb = 0, mz[4] = {0, 0, 0, 0};
                        for (int k = 0; k < G.nn - 1; k++) {
                            const int s = G.nodes[k];
                            if (G.missing(G.par[s])) continue;
                            mz[2 * (G.missing(s) ? 1 : 0) + (G.Z[s] == 1 ? 1 : 0)] += 1;
                            if (G.missing(s)) continue;
                            if (G.B[s]) gb++; else ungb++;
                        }
                        f += sc.lmis[0] * mz[0] + sc.lmis[1] * mz[1] + sc.lmis[2] * mz[2] + sc.lmis[3] * mz[3];
                        f += sc.ec_gc[0] * ungb + lgpdf(sc.r_gb, p.gca, p.gcb, sc.pr_lg[2], sc.pr_alb[2]) +
                             sc.ec_gc[1] * gb;
                        sc.full = f;
                    }
                    trd[0 * p.T + m] = sc.full;
                    trd[1 * p.T + m] = sc.r_n;
                    trd[2 * p.T + m] = sc.r_c;
                    trd[3 * p.T + m] = sc.r_gb;
                    sc.changed = (m >= p.burn && sc.full > sc.MaxLoglik) ? 1 : 0;
                    if (sc.changed) sc.MaxLoglik = sc.full;
                }
                __syncthreads();
                for (int s = tid; s < N; s += blockDim.x) {
                    trzb[((size_t)m * 2) * p.N_max + s] = G.Z[s];
                    trzb[((size_t)m * 2 + 1) * p.N_max + s] = G.B[s];
                    if (sc.changed) { G.MZ[s] = G.Z[s]; G.MB[s] = G.B[s]; }
                }
                if (m == p.T - 1) break;
                __syncthreads();
                GB_MARK(0)
                // expected counts of the accepted partials
                if (sc.move_r) {
                    const int nx = 1 - sc.post_cur;
                    counts(p, G, sc.pbuf, G.post + (size_t)nx * N * 16);
                    GB_MARK(1)
                    if (tid == 0) sc.post_nxt = nx;
                    __syncthreads();
                }
                if (m == 0) {
                    if (tid == 0) sc.post_cur = sc.post_nxt;
                    __syncthreads();
                }
                const Real* post = G.post + (size_t)sc.post_cur * N * 16;
                // initial_prob_back
                emissions(G, sc, G.emis, 0, sc.cur, post, true);
                if (tid == 0) {
                    double el = 0;
                    for (int k = 0; k < G.nn - 1; k++) {
                        const int s = G.nodes[k];
                        if (!G.missing(s)) el += G.eraw[s];
                    }
                    sc.elbo_old = el;
                }
                prob_back(G, sc, G.emis);
                if (tid == 0) {
                    sc.loglik_old = lpb_root(G);
                    sc.acc = sc.cur;
                }
                for (int i = tid; i < N * 6; i += blockDim.x) G.emis_tmp[i] = G.emis[i];
                __syncthreads();
                GB_MARK(2)
                // sample_rates: three MH moves of (gB, n, c) with Z and B integrated out
                if (tid == 0) {
                    sc.x_gb = sc.r_gb; sc.x_n = sc.r_n; sc.x_c = sc.r_c;
                    // the current values' terms of the MH ratio, computed once
                    // and carried over to an accepted proposal's
                    sc.lg_x[0] = lgpdf(sc.x_gb, p.gca, p.gcb, sc.pr_lg[2], sc.pr_alb[2]);
                    sc.lg_x[1] = resZ != 0 ? lgpdf(__dadd_rn(sc.x_n, p.nshift), p.na, p.nb, sc.pr_lg[1], sc.pr_alb[1]) : 0.0;
                    sc.lg_x[2] = lgpdf(-sc.x_c, p.ca, p.cb, sc.pr_lg[0], sc.pr_alb[0]);
                    sc.lg_x[3] = d_log(-sc.x_c);
                }
                for (int mm = 0; mm < 3; mm++) {
                    __shared__ double cur3[3];
                    if (tid == 0) {
                        // cur3: the chain's values (the last accepted proposal); x_*: the new proposal
                        cur3[0] = sc.x_gb; cur3[1] = sc.x_n; cur3[2] = sc.x_c;
                        double u = __dmul_rn(__dmul_rn(__dsub_rn(rng.uniform(), 0.5), p.prop_gc), 2.0);
                        double ngb = __dadd_rn(cur3[0], u);
                        if (ngb < 0.01) ngb = cur3[0];
                        double nn_ = cur3[1];
                        if (resZ != 0) {
                            const double inv = __ddiv_rn(1.0, p.prop_n);
                            u = __dadd_rn(__dmul_rn(rng.uniform(), __dsub_rn(p.prop_n, inv)), inv);
                            nn_ = __dsub_rn(__dmul_rn(__dadd_rn(cur3[1], p.nshift), u), p.nshift);
                        }
                        const double invc = __ddiv_rn(1.0, p.prop_c);
                        u = __dadd_rn(__dmul_rn(rng.uniform(), __dsub_rn(p.prop_c, invc)), invc);
                        const double nc_ = __dmul_rn(cur3[2], u);
                        sc.sel[0] = nc_; sc.sel[1] = nn_; sc.sel[2] = 0.0; sc.sel[3] = nc_; sc.sel[4] = nn_;
                        sc.bias[0] = 0.0; sc.bias[1] = 0.0; sc.bias[2] = ngb; sc.bias[3] = ngb; sc.bias[4] = ngb;
                        int pr = 0;
                        while (pr == sc.cur || pr == sc.acc) pr++;
                        sc.prop = pr;
                    }
                    __syncthreads();
                    {
                        const int cls[5] = {1, 2, 3, 4, 5};
                        build_caches(p, G, 5, cls, sc.sel, sc.bias, sc.prop);
                    }
                    GB_MARK(3)
                    emissions(G, sc, G.emis_tmp, 1, sc.prop, post, false);
                    prob_back(G, sc, G.emis_tmp);
                    if (tid == 0) {
                        const double lr = lpb_root(G);
                        const double ngb = sc.bias[2], nn_ = sc.sel[1], nc_ = sc.sel[0];
                        // the proposal's terms; the current values' are in lg_x
                        const double ly[4] = {
                            lgpdf(ngb, p.gca, p.gcb, sc.pr_lg[2], sc.pr_alb[2]),
                            resZ != 0 ? lgpdf(__dadd_rn(nn_, p.nshift), p.na, p.nb, sc.pr_lg[1], sc.pr_alb[1]) : 0.0,
                            lgpdf(-nc_, p.ca, p.cb, sc.pr_lg[0], sc.pr_alb[0]), d_log(-nc_)};
                        double MH = __dsub_rn(__dadd_rn(__dsub_rn(lr, sc.loglik_old), ly[0]), sc.lg_x[0]);
                        if (resZ != 0) MH = __dadd_rn(MH, __dsub_rn(ly[1], sc.lg_x[1]));
                        MH = __dadd_rn(MH, __dadd_rn(__dsub_rn(__dsub_rn(ly[2], sc.lg_x[2]), ly[3]), sc.lg_x[3]));
                        const bool acc = d_log(rng.uniform()) < MH;
                        sc.changed = acc ? 1 : 0;
                        if (acc) {
                            sc.x_gb = ngb; sc.x_n = nn_; sc.x_c = nc_;
                            for (int q = 0; q < 4; q++) sc.lg_x[q] = ly[q];
                            sc.loglik_old = lr;
                            sc.acc = sc.prop;
                        }
                    }
                    __syncthreads();
                    const bool accepted = sc.changed;
                    for (int i = tid; i < (G.nn - 1) * 5; i += blockDim.x) {
                        const int s = G.nodes[i / 5], j = 1 + i % 5;
                        if (G.missing(s) || (G.fixZ[s] == 1 && j % 3 == 2)) continue;
                        if (accepted) G.emis[s * 6 + j] = G.emis_tmp[s * 6 + j];
                        else G.emis_tmp[s * 6 + j] = G.emis[s * 6 + j];
                    }
                    __syncthreads();
                    GB_MARK(4)
                }
                // update_rates: Update_ZB, a pruning pass, ELBO, one MH step
                for (int s = tid; s < N; s += blockDim.x) { G.Zp[s] = G.Z[s]; G.Bp[s] = G.B[s]; }
                if (tid == 0) sc.changed = 0;
                prob_back(G, sc, G.emis);
                if (tid == 0) sc.pos = rng.pos;
                __syncthreads();
                sample_zb(p, G, sc);
                GB_MARK(5)
                stage_pcur(G, sc.acc);
                prune(p, G, sc, 1 - sc.pbuf);
                GB_MARK(6)
                for (int k = tid; k < G.nn - 1; k += blockDim.x) {
                    const int s = G.nodes[k];
                    if (G.missing(s)) continue;
                    const Real* a2 = G.lp(G.slot(G.Z[s] + 3 * G.B[s], sc.acc), s);
                    const Real* b2 = post + (size_t)s * 16;
                    Real t = 0;
                    for (int c = 0; c < 4; c++)
                        for (int r = 0; r < 4; r++) t += a2[r * 4 + c] * b2[r * 4 + c];
                    G.eraw[s] = (double)t;
                }
                __syncthreads();
                if (tid == 0) {
                    rng.pos += (uint64_t)(G.nn - 1);
                    double elbo_new = 0;
                    for (int k = 0; k < G.nn - 1; k++) {
                        const int s = G.nodes[k];
                        if (!G.missing(s)) elbo_new += G.eraw[s];
                    }
                    const double MH = __dsub_rn(__dadd_rn(__dsub_rn(sc.colsum, sc.tl), sc.elbo_old), elbo_new);
                    if (d_log(rng.uniform()) < MH) {
                        sc.tl_next = sc.colsum;
                        if (sc.changed) sc.logp_Z = prior_z(G, sc) - sc.logpZC;
                        sc.cur = sc.acc;
                        sc.pbuf = 1 - sc.pbuf;
                        sc.r_gb = sc.x_gb; sc.r_n = sc.x_n; sc.r_c = sc.x_c;
                        sc.move_r = 1;
                    } else {
                        sc.move_r = 0;
                    }
                    sc.post_cur = sc.post_nxt;
                }
                __syncthreads();
                if (!sc.move_r)
                    for (int s = tid; s < N; s += blockDim.x) { G.Z[s] = G.Zp[s]; G.B[s] = G.Bp[s]; }
                __syncthreads();
                GB_MARK(7)
            }
            __syncthreads();
            if (tid == 0) p.max_ll[(size_t)e * 3 + resZ] = sc.MaxLoglik;
            for (int s = tid; s < N; s += blockDim.x) {
                p.max_zb[(((size_t)e * 3 + resZ) * 2) * p.N_max + s] = G.MZ[s];
                p.max_zb[(((size_t)e * 3 + resZ) * 2 + 1) * p.N_max + s] = G.MB[s];
            }
            __syncthreads();
        }
        if (tid == 0) {
            p.status[e] = 0;
            if (p.phase)
                for (int q = 0; q < 8; q++) atomicAdd(&p.phase[q], s_ph[q]);
        }
        if (p.stream) {
            // publish the slot once every thread's output writes are visible
            __threadfence_system();
            __syncthreads();
            if (tid == 0) p.done_flag[e] = 1;
        }
        __syncthreads();
    }
}

// Dynamic shared memory of the chain kernel for N nodes.
size_t gbgc_chain_smem(int N, int prec) {
    const size_t rb = prec ? 4 : 8;
    size_t o = (size_t)N * 16 * rb + 5 * 13 * 16 * 8 + 8 * 8;
    o += ((size_t)6 * N + 4 * (size_t)N + 4) * 2 + (size_t)4 * N;
    o = (o + 15) & ~(size_t)15;
    o += (size_t)8 * N;
    return o;
}

int gbgc_chain_threads() { return GB_BT; }
int gbgc_chain_warps() { return GB_WARPS; }

// Register budgets: 168 (3 CTAs an SM) or 96 (5 CTAs an SM, some spills).
template <typename Real, int MINB>
static cudaError_t launch_one(const GbgcChainParams& p, int grid, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(gbgc_chain_kernel<Real, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    gbgc_chain_kernel<Real, MINB><<<grid, GB_BT, smem, st>>>(p);
    return cudaGetLastError();
}

int gbgc_chain_occupancy(int prec, int regs, size_t smem) {
    int n = 0;
    cudaError_t e;
    if (regs == 168)
        e = prec ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gbgc_chain_kernel<float, 3>, GB_BT, smem)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gbgc_chain_kernel<double, 3>, GB_BT, smem);
    else
        e = prec ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gbgc_chain_kernel<float, 5>, GB_BT, smem)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gbgc_chain_kernel<double, 5>, GB_BT, smem);
    return e == cudaSuccess ? n : 0;
}

cudaError_t launch_gbgc_chain(const GbgcChainParams& p, int grid, size_t smem, int prec, int regs, cudaStream_t st) {
    if (regs == 168) return prec ? launch_one<float, 3>(p, grid, smem, st) : launch_one<double, 3>(p, grid, smem, st);
    return prec ? launch_one<float, 5>(p, grid, smem, st) : launch_one<double, 5>(p, grid, smem, st);
}

}  // namespace pacc
