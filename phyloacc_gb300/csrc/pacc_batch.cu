// pacc_batch.cu — the batched, resumable chain kernel: one warp per element
// chain, many chains per SM, chain state resident in device memory between
// launches.
//
// Same sampler as pacc_chain.cu (PhyloAcc-ST's initMCMC -> Gibbs -> Eval2 ->
// Output_init for M0, M1, M2; src/PhyloAcc-ST/main.cpp:468-494) with a
// layout built for many concurrent chains:
//   * a chain is a warp; a CTA holds several chains, each with its own slice
//     of shared memory and its own position in the element queue;
//   * partial likelihoods are never stored between steps: every pass over the
//     columns recomputes them column by column in a per-lane shared-memory
//     slice (one column per lane), so the only per-iteration device-memory
//     traffic is the element's column codes.  The reference's partial
//     re-pruning (bpp_c.cpp:620-642) is an optimisation over stored partials
//     and gives the same values as a full prune;
//   * the internal-base pass samples, and counts the (child, parent) base
//     pairs that the branch emissions need (getEmission, bpp_c2.cpp:355-390),
//     in the same sweep over a column;
//   * the latent-state filter runs in linear space in FP64 with per-node
//     normalisation (the reference's log-space log_multi2, bpp.hpp:447-460,
//     computes the same messages);
//   * a launch advances each resident chain by a bounded number of iterations
//     and saves its state, so a host loop can retire finished chains and admit
//     new ones between launches (serving), and a fixed launch sequence can be
//     captured in a CUDA graph.
// Real = float: FP32 partials with power-of-two rescaling folded into one
// integer exponent per column; per-column log-likelihoods are combined in
// FP64 (mantissa products + exact exponents); exp(lambda*r*t), the MH ratio,
// the Z filter normalisation and the chain scalars stay in FP64.
// Real = double: the same kernel in FP64, used to check this layout against
// the oracle draw for draw.
#include "pacc_common.cuh"

namespace pacc {

// Per-slot device workspace.
struct SlotLayout {
    size_t Z, maxz, tbl, trz, trd, total;
    __host__ __device__ static SlotLayout make(int N, int T) {
        SlotLayout L;
        size_t o = 0;
        auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
        L.Z = o; o = al(o + N);
        L.maxz = o; o = al(o + N);
        L.tbl = o; o = al(o + (size_t)3 * N * 16 * 8);     // class P^T tables, FP64 [null, cons, neut][N][16]
        L.trz = o; o = al(o + (size_t)T * N);
        L.trd = o; o = al(o + (size_t)7 * T * 8);
        L.total = o;
        return L;
    }
};

// Per-warp Eval2 scratch.
struct GrpLayout {
    size_t hash, rep, cfg, nxt, head, first, cstat, pst, amb, total;
    __host__ __device__ static GrpLayout make(int mcmc, int NI, int real_bytes, int GGuP, int NZ) {
        GrpLayout L;
        size_t o = 0;
        auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
        // the chain's internal partials per site pattern, two buffers (current
        // state / proposal): [2][NI][GGuP][4]
        L.pst = o; o = al(o + (size_t)2 * NI * GGuP * 4 * real_bytes);
        L.amb = o; o = al(o + (size_t)NZ * 24 * 4);        // (ambiguity code, parent base) counts of leaves
        L.hash = o; o = al(o + (size_t)(mcmc + 1) * 8);
        L.rep = o; o = al(o + (size_t)(mcmc + 1) * 4);
        L.cfg = o; o = al(o + (size_t)(mcmc + 1) * 4);
        L.nxt = o; o = al(o + (size_t)(mcmc + 1) * 4);
        L.head = o; o = al(o + (size_t)(mcmc + 2) * 4);
        L.first = o; o = al(o + (size_t)(mcmc + 2) * 4);
        L.cstat = o; o = al(o + (size_t)9 * (mcmc + 2) * 8);
        L.total = o;
        return L;
    }
};

// Shared memory of one warp-chain; every lane carries C columns.
template <typename Real>
struct WarpSmem {
    size_t ptc, part, tgv, rec, srec, stage, cnt, topo, i8, dbl, total;
    __host__ __device__ static WarpSmem make(int N, int NI, int S, int D, int C) {
        WarpSmem w;
        size_t o = 0;
        auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
        w.ptc = o; o = al(o + (size_t)N * 16 * sizeof(Real));        // current P^T per branch
        size_t part_bytes = (size_t)D * C * 4 * 32 * sizeof(Real);      // stack of pending partials
        size_t alias_bytes = (size_t)N * 6 * 8;                        // emissions + Z filter alias the stack
        w.part = o; o = al(o + (part_bytes > alias_bytes ? part_bytes : alias_bytes));
        w.tgv = o; o = al(o + (size_t)NI * C * 32);
        w.rec = o; o = al(o + (size_t)NI * sizeof(NodeRec));
        w.srec = o; o = al(o + (size_t)NI * sizeof(NodeRec));
        w.stage = o; o = al(o + (size_t)C * ((S + 15) & ~15) * 32);
        w.cnt = o; o = al(o + (size_t)N * 16 * 2);                      // uint16 bins (base, parent base)
        w.topo = o; o = al(o + (size_t)TopoLayout::make(N).total * 2);
        w.i8 = o; o = al(o + (size_t)N * 6);                            // fixZ chg unv mask (unused) Z
        w.dbl = o; o = al(o + (size_t)N * 8);                           // branch lengths of the pruned tree
        w.total = o;
        return w;
    }
};

// ---------------------------------------------------------------------------
// per-warp context
// ---------------------------------------------------------------------------
template <typename Real, int C>
struct W {
    int lane, S, N, GG, GGp, root, n_nodes, n_int, n_hlev, n_dlev, tg_draws, T, burn, mcmc;
    const uint8_t* codes;
    const int32_t* prefix;
    int16_t *nodes, *internal, *c2a, *c2b, *par, *irank, *pos, *missing, *upc, *upcc, *hlev_start, *hlev_nodes,
        *dlev_start, *dlev_nodes;
    Real* ptc;          // [N][16]
    Real* part;         // stack of pending partials [D][C][4][32]
    int8_t* tgv;        // [NI][C][32] sampled base (or 4: no data) per internal node and column
    const NodeRec* rec; // [NI] internal nodes in postorder (internal_nodes)
    const NodeRec* srec;// [NI] internal nodes in stack order
    Real* pst[2];       // per-warp device scratch [2][NI][GGuP][4]: partials per pattern, by buffer
    int GGuP;           // pattern stride of pst
    int n_int_max;      // row count of pst
    int cur;            // buffer of pst that holds the current state's partials
    const int32_t* pof; // [GG] pattern of each column
    uint32_t* stage;    // [C][SP/4][32] words of per-lane column codes
    const uint8_t* codes_t;  // [GGp][SP]
    const uint8_t* pcodes_t; // [GGu rounded up to 32][SP] site patterns
    const int32_t* pw;       // [GGu] pattern weights
    int GGu;
    int SP;
    unsigned* cnt;      // [N][8] packed uint16 pairs: (base, parent base) counts per branch
    unsigned* amb;      // [N][24] (ambiguity code, parent base) counts of leaf branches (device memory)
    double* emis;       // [N][3]  (aliases part)
    double* bz;         // [N][3]  (aliases part)
    double* dist2;      // [N]
    int8_t *Z, *fixZ, *chg, *unv, *mask;
    // slot workspace
    int8_t* sZ;
    int8_t* smaxz;
    double* tbl;        // [3][N][16]
    int8_t* trz;        // [T][N]
    double* trd;        // [7][T]
    SlotState st;       // lane-replicated copy
    unsigned long long e_int, e_leaf, n_tg;
    unsigned long long ph[8];
    long long t0;

    __device__ __forceinline__ Real& P(int s, int i, int j) { return ptc[s * 16 + i * 4 + j]; }
};

__device__ __forceinline__ void wsync() { __syncwarp(); }

// 4-state vectors and 4x4 matrices move as 16-byte accesses: a partial of
// lane l lives at [.. * 32 + l][4], a matrix row-major in 16 contiguous words.
__device__ __forceinline__ void ld4(const float* __restrict__ p, float (&x)[4]) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
}
__device__ __forceinline__ void ld4(const double* __restrict__ p, double (&x)[4]) {
    const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
    x[0] = a.x; x[1] = a.y; x[2] = b.x; x[3] = b.y;
}
__device__ __forceinline__ void st4(float* __restrict__ p, const float (&x)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(x[0], x[1], x[2], x[3]);
}
__device__ __forceinline__ void st4(double* __restrict__ p, const double (&x)[4]) {
    reinterpret_cast<double2*>(p)[0] = make_double2(x[0], x[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(x[2], x[3]);
}
template <typename Real>
__device__ __forceinline__ void ld16(const Real* __restrict__ p, Real (&m)[16]) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
        Real t[4];
        ld4(p + 4 * r, t);
#pragma unroll
        for (int i = 0; i < 4; i++) m[4 * r + i] = t[i];
    }
}


// Phase timer of a warp (lane 0): cycles since the previous mark go to phase i.
#define PHASE(i)                               \
    do {                                       \
        if (w.lane == 0) {                     \
            long long t_ = clock64();          \
            w.ph[i] += (unsigned long long)(t_ - w.t0); \
            w.t0 = t_;                         \
        }                                      \
    } while (0)

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int warp_or(int v) { return __any_sync(0xffffffffu, v); }

enum { TR_LL = 0, TR_FULL = 1, TR_N = 2, TR_C = 3, TR_G = 4, TR_L = 5, TR_L2 = 6 };
enum { C_NULL = 0, C_CONS = 1, C_NEUT = 2 };

// Fill the current per-branch matrices: class by Z (null / cons / neut,
// bpp_c.cpp:661-663); with prop_class >= 0 the branches of that class get the
// proposal matrices P(d * r_prop) (log_f_Xz, bpp_c.cpp:885-906).
template <typename Real, int C>
__device__ __noinline__ void fill_ptc(W<Real, C>& w, int prop_class, double r_prop) {
    // branches that take a class table: one matrix row (4 words) per lane and
    // step, so that consecutive lanes write consecutive 16-byte chunks
    const int nb = w.n_nodes - 1;
    for (int idx = w.lane; idx < nb * 4; idx += 32) {
        const int s = w.nodes[idx >> 2], row = idx & 3;
        const int z = w.Z[s];
        const int k = (z == 2) ? C_NEUT : (z == 0 ? C_NULL : C_CONS);
        if (prop_class >= 0 && k == prop_class) continue;
        const double* src = w.tbl + ((size_t)k * w.N + s) * 16 + row * 4;
        const Real v[4] = {(Real)src[0], (Real)src[1], (Real)src[2], (Real)src[3]};
        st4(w.ptc + s * 16 + row * 4, v);
    }
    // branches of the proposal class: P(d * r_prop) built per lane
    if (prop_class >= 0) {
        for (int i = w.lane; i < nb; i += 32) {
            const int s = w.nodes[i];
            const int z = w.Z[s];
            const int k = (z == 2) ? C_NEUT : (z == 0 ? C_NULL : C_CONS);
            if (k != prop_class) continue;
            double pt[16];
            build_pt(w.dist2[s], r_prop, true, pt);
            for (int q = 0; q < 16; q++) w.ptc[s * 16 + q] = (Real)pt[q];
        }
    }
    wsync();
}

// Class table k at rate r for all branches of the pruned tree; branches not
// longer than 1e-10 keep the identity (bpp_c.cpp:191-226) unless force.
template <typename Real, int C>
__device__ __noinline__ void build_table(W<Real, C>& w, int k, double r, bool scaled, bool force, bool skip_short) {
    for (int i = w.lane; i < w.n_nodes - 1; i += 32) {
        int s = w.nodes[i];
        double* out = w.tbl + ((size_t)k * w.N + s) * 16;
        if (skip_short && w.dist2[s] < 1e-10) continue;
        if (force || w.dist2[s] > 1e-10) build_pt(w.dist2[s], r, scaled, out);
        else identity_pt(out);
    }
    wsync();
}

template <typename Real> struct Resc;
template <> struct Resc<double> {
    static __device__ __forceinline__ void apply(double* a, int& sc) {
        double mx = fmax(fmax(a[0], a[1]), fmax(a[2], a[3]));
        if (mx < 0x1p-256 && mx > 0) {
            do {
                for (int j = 0; j < 4; j++) a[j] *= 0x1p256;
                sc -= 256;
                mx *= 0x1p256;
            } while (mx < 0x1p-256);
        }
    }
};
template <> struct Resc<float> {
    static __device__ __forceinline__ void apply(float* a, int& sc) {
        float mx = fmaxf(fmaxf(a[0], a[1]), fmaxf(a[2], a[3]));
        if (mx < 0x1p-40f && mx > 0) {
            int e;
            frexpf(mx, &e);
            int k = -e;   // scale the max into [0.5, 1)
            float f1 = ldexpf(1.0f, k / 2), f2 = ldexpf(1.0f, k - k / 2);
            for (int j = 0; j < 4; j++) a[j] = (a[j] * f1) * f2;
            sc -= k;
        }
    }
};

// Load the codes of column g of every taxon into this lane's stage words:
// the column is SP contiguous bytes (codes by column), read with SP/16
// independent 128-bit loads.  Stage layout: word ((c >> 2) * 32 + lane) holds
// taxa c..c+3 of this lane's column.
__device__ __forceinline__ void stage_column(const uint8_t* __restrict__ codes_t, int SP, uint32_t* __restrict__ stage,
                                             int lane, int g, bool act) {
    const int nv = SP >> 4;
    if (act) {
        const uint4* __restrict__ src = (const uint4*)(codes_t + (size_t)g * SP);
        for (int i0 = 0; i0 < nv; i0 += 4) {   // up to 4 loads in flight (64 taxa)
            uint4 v[4];
#pragma unroll
            for (int i = 0; i < 4; i++)
                if (i0 + i < nv) v[i] = src[i0 + i];
#pragma unroll
            for (int i = 0; i < 4; i++)
                if (i0 + i < nv) {
                    const int b = 4 * (i0 + i);
                    stage[(b + 0) * 32 + lane] = v[i].x;
                    stage[(b + 1) * 32 + lane] = v[i].y;
                    stage[(b + 2) * 32 + lane] = v[i].z;
                    stage[(b + 3) * 32 + lane] = v[i].w;
                }
        }
    } else {
        for (int i = 0; i < 4 * nv; i++) stage[i * 32 + lane] = 0x04040404u;  // gaps
    }
}

__device__ __forceinline__ int stage_code(const uint32_t* __restrict__ stage, int c, int lane) {
    return (stage[(c >> 2) * 32 + lane] >> (8 * (c & 3))) & 0xFF;
}

// Bottom-up pass over the C columns held by this lane (Update_Tg without
// sampling, bpp_c.cpp:647-671); column j of the lane is stage set j.  Internal
// nodes are visited in stack order (a postorder that takes the child needing
// more pending partials first); a node pops its internal children's partials
// and pushes its own, so at most `stack_depth` partials per column are live.
// The C columns share every node record and every matrix load, and their
// arithmetic is independent, which hides the latency of each.  The "has
// data" flag of a node (some leaf below is a base or an ambiguity code: the
// complement of Tg == K, bpp_c.hpp:417-428) travels on a register bit stack
// per column.  With STORE, every partial is also written to the chain's
// partial buffer (rows by internal rank, columns by pattern g0 + 32 j + lane)
// for the top-down sampling.
// sc[j] gets the rescale exponent of column j and root[j] its root partial
// (pi included).
template <typename Real, int C, bool STORE>
__device__ __forceinline__ void column_up(const NodeRec* __restrict__ srec, int n_int,
                                          const uint32_t* __restrict__ stage, int sstride, Real* __restrict__ stk,
                                          Real* __restrict__ pout, int GGuP, int g0,
                                          const Real* __restrict__ ptc, int lane, const bool (&act)[C],
                                          unsigned& e_int, unsigned& e_leaf, const Real pi[4], Real (&root)[C][4],
                                          int (&sc)[C]) {
    int sp = 0;
    unsigned hbits[C];
#pragma unroll
    for (int j = 0; j < C; j++) { hbits[j] = 0; sc[j] = 0; }
    for (int k = 0; k < n_int; k++) {
        const NodeRec R = srec[k];
        const bool i0 = R.r0 >= 0, i1 = R.r1 >= 0;
        Real x0[C][4], x1[C][4];
        bool h0[C], h1[C];
        int code0[C], code1[C];
        // pop internal children (the child computed last is on top)
        if (i0 && i1) {
            const bool c0_top = R.prank & 1;   // flags, see NodeRec
            const Real* t = stk + (sp - 1) * (C * 128) + lane * 4;
            const Real* u = stk + (sp - 2) * (C * 128) + lane * 4;
            sp -= 2;
#pragma unroll
            for (int j = 0; j < C; j++) {
                const bool ht = hbits[j] & 1, hu = (hbits[j] >> 1) & 1;
                hbits[j] >>= 2;
                Real tt[4], uu[4];
                ld4(t + j * 128, tt);
                ld4(u + j * 128, uu);
#pragma unroll
                for (int i = 0; i < 4; i++) { x0[j][i] = c0_top ? tt[i] : uu[i]; x1[j][i] = c0_top ? uu[i] : tt[i]; }
                h0[j] = c0_top ? ht : hu;
                h1[j] = c0_top ? hu : ht;
            }
        } else if (i0 || i1) {
            const Real* t = stk + (sp - 1) * (C * 128) + lane * 4;
            sp -= 1;
#pragma unroll
            for (int j = 0; j < C; j++) {
                const bool ht = hbits[j] & 1;
                hbits[j] >>= 1;
                ld4(t + j * 128, x0[j]);
#pragma unroll
                for (int i = 0; i < 4; i++) x1[j][i] = x0[j][i];
                h0[j] = ht;
                h1[j] = ht;
            }
        }
#pragma unroll
        for (int j = 0; j < C; j++) {
            code0[j] = 0;
            code1[j] = 0;
            if (!i0) { code0[j] = stage_code(stage + j * sstride, R.c0, lane); h0[j] = code0[j] != CODE_GAP && code0[j] != CODE_OTHER; }
            if (!i1) { code1[j] = stage_code(stage + j * sstride, R.c1, lane); h1[j] = code1[j] != CODE_GAP && code1[j] != CODE_OTHER; }
        }
        Real a[C][4];
        bool hs[C];
#pragma unroll
        for (int j = 0; j < C; j++) {
            hs[j] = h0[j] || h1[j];
#pragma unroll
            for (int i = 0; i < 4; i++) a[j][i] = 1;
        }
        if (!R.missing) {
#pragma unroll
            for (int q = 0; q < 2; q++) {
                if (q ? R.m1 : R.m0) continue;
                const int c = q ? R.c1 : R.c0;
                const Real* __restrict__ Pc = ptc + c * 16;
                if (q ? i1 : i0) {
                    // internal child: one matrix load serves all C columns
                    Real p[16];
                    ld16(Pc, p);
#pragma unroll
                    for (int j = 0; j < C; j++) {
                        const Real* x = q ? x1[j] : x0[j];
                        const bool use = act[j] && hs[j] && (q ? h1[j] : h0[j]);
                        const Real d0 = (p[0] * x[0] + p[4] * x[1]) + (p[8] * x[2] + p[12] * x[3]);
                        const Real d1 = (p[1] * x[0] + p[5] * x[1]) + (p[9] * x[2] + p[13] * x[3]);
                        const Real d2 = (p[2] * x[0] + p[6] * x[1]) + (p[10] * x[2] + p[14] * x[3]);
                        const Real d3 = (p[3] * x[0] + p[7] * x[1]) + (p[11] * x[2] + p[15] * x[3]);
                        if (use) {
                            a[j][0] *= d0; a[j][1] *= d1; a[j][2] *= d2; a[j][3] *= d3;
                            e_int++;
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < C; j++) {
                        const int code = q ? code1[j] : code0[j];
                        if (!(act[j] && hs[j] && (q ? h1[j] : h0[j]))) continue;
                        if (code < 4) {
                            Real pr[4];
                            ld4(Pc + code * 4, pr);
                            a[j][0] *= pr[0]; a[j][1] *= pr[1]; a[j][2] *= pr[2]; a[j][3] *= pr[3];
                        } else {
                            int msk = ambig_mask(code - CODE_R);
                            Real v0 = 0, v1 = 0, v2 = 0, v3 = 0;
#pragma unroll
                            for (int i = 0; i < 4; i++)
                                if (msk & (1 << i)) { v0 += Pc[i * 4]; v1 += Pc[i * 4 + 1]; v2 += Pc[i * 4 + 2]; v3 += Pc[i * 4 + 3]; }
                            a[j][0] *= v0; a[j][1] *= v1; a[j][2] *= v2; a[j][3] *= v3;
                        }
                        e_leaf++;
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < C; j++)
                if (act[j] && hs[j]) Resc<Real>::apply(a[j], sc[j]);
        }
        Real* __restrict__ o = stk + sp * (C * 128) + lane * 4;
        sp++;
#pragma unroll
        for (int j = 0; j < C; j++) {
            if (R.is_root) {
#pragma unroll
                for (int i = 0; i < 4; i++) { a[j][i] *= pi[i]; root[j][i] = a[j][i]; }
            }
            st4(o + j * 128, a[j]);
            hbits[j] = (hbits[j] << 1) | (hs[j] ? 1u : 0u);
            if (STORE && act[j]) {
                // a node without data below it (other than the root, which is
                // always drawn) is kept as (-1,-1,-1,-1): the sampling pass
                // reads the mark with the partial
                const size_t at = (size_t)R.self * GGuP + g0 + 32 * j + lane;
                if (hs[j] || R.is_root) st4(pout + at * 4, a[j]);
                else {
                    const Real m[4] = {-1, -1, -1, -1};
                    st4(pout + at * 4, m);
                }
            }
        }
    }
}

// Per-column log-likelihood accumulated as (FP64 product of root sums) x 2^exponent.
struct LLAcc {
    double prod;
    long long e2;
    double lsum;   // weighted site patterns: FP64 sum of w log(mantissa)
    __device__ void init() { prod = 1.0; e2 = 0; lsum = 0; }
    __device__ void add_weighted(double t, int sc, int wgt) {
        int e;
        const double m = frexp(t, &e);
        lsum += (double)wgt * d_log(m);
        e2 += (long long)wgt * (e + sc);
    }
    __device__ void add(double t, int sc) {
        int e;
        double m = frexp(t, &e);
        prod *= m;
        e2 += e + sc;
        int e3;
        prod = frexp(prod, &e3);
        e2 += e3;
    }
    __device__ double value() const { return d_log(prod) + lsum + (double)e2 * 0.6931471805599453; }
};

// Full prune with the current matrices; returns the summed per-column
// log-likelihood (log_exp_sum at the root, bpp_c.cpp:429).  The pass runs over
// the element's site patterns and weights each pattern by its column count.
// A pass covers 32 x C patterns: lane l takes patterns g0 + 32 j + l.  Every
// internal partial is kept in partial buffer buf (0 or 1; the reference
// keeps lambda / lambda_tmp the same way, bpp_c.cpp:981-989,1115).
template <typename Real, int C>
__device__ __noinline__ double likelihood_pass(W<Real, C>& w, int buf) {
    const int lane = w.lane, n_int = w.n_int, GU = w.GGu, SP = w.SP;
    const int sstride = (SP >> 2) * 32;
    const NodeRec* __restrict__ srec = w.srec;
    const uint8_t* __restrict__ codes_t = w.pcodes_t;
    const int32_t* __restrict__ pw = w.pw;
    uint32_t* __restrict__ stage = w.stage;
    Real* __restrict__ stk = w.part;
    const Real* __restrict__ ptc = w.ptc;
    Real* __restrict__ pout = w.pst[buf];
    const int GGuP = w.GGuP;
    const Real pi[4] = {(Real)dM.pi[0], (Real)dM.pi[1], (Real)dM.pi[2], (Real)dM.pi[3]};
    unsigned e_int = 0, e_leaf = 0;
    double acc = 0;
    LLAcc ll;
    ll.init();
    for (int g0 = 0; g0 < GU; g0 += 32 * C) {
        bool act[C];
#pragma unroll
        for (int j = 0; j < C; j++) {
            const int g = g0 + 32 * j + lane;
            act[j] = g < GU;
            stage_column(codes_t, SP, stage + j * sstride, lane, g, act[j]);
        }
        Real r[C][4];
        int sc[C];
        column_up<Real, C, true>(srec, n_int, stage, sstride, stk, pout, GGuP, g0, ptc, lane, act, e_int, e_leaf,
                                 pi, r, sc);
#pragma unroll
        for (int j = 0; j < C; j++) {
            if (act[j]) {
                const int wgt = pw[g0 + 32 * j + lane];
                double t = (double)r[j][0] + (double)r[j][1] + (double)r[j][2] + (double)r[j][3];
                if (sizeof(Real) == 8) acc += (double)wgt * (d_log(t) + (double)sc[j] * 0.6931471805599453);
                else if (wgt == 1) ll.add(t, sc[j]);
                else ll.add_weighted(t, sc[j], wgt);
            }
        }
    }
    w.e_int += e_int;
    w.e_leaf += e_leaf;
    double v = (sizeof(Real) == 8) ? acc : ll.value();
    return warp_sum(v);
}

// Inverse-CDF categorical draw in the partials' precision.
template <typename Real>
__device__ __forceinline__ int cat4(const Real* p, double u) {
    if (sizeof(Real) == 8) return categorical(4, p, u);
    float tot = ((float)p[0] + (float)p[1]) + ((float)p[2] + (float)p[3]);
    float t = (float)u * tot;
    float cum = 0;
    for (int k = 0; k < 4; k++) {
        cum += (float)p[k];
        if (t < cum) return k;
    }
    for (int k = 3; k >= 0; k--)
        if (p[k] > 0) return k;
    return 4;
}

// Uniform from a stream word in the partials' precision.
template <typename Real>
__device__ __forceinline__ double u_of(uint32_t w) { return word_to_uniform(w); }
template <>
__device__ __forceinline__ double u_of<float>(uint32_t w) {
    return (double)(((float)(w >> 8) + 0.5f) * 5.9604644775390625e-08f);
}

// Internal-base pass (Update_Tg with sampling, bpp_c.cpp:672-733) fused with
// the emission histogram.  The partials are those of the current state, kept
// by the last likelihood pass in buffer w.cur (per site pattern); column g
// reads the row of its pattern.  Each column draws from its own words of the
// stream (prefix[g] words before it), so the draws do not depend on how
// columns are spread over lanes.
template <typename Real, int C>
__device__ __noinline__ int sample_pass(W<Real, C>& w, uint64_t pos) {
    const int lane = w.lane, n_int = w.n_int, GG = w.GG, SP = w.SP, N = w.N;
    const int sstride = (SP >> 2) * 32;
    const NodeRec* __restrict__ rec = w.rec;
    const uint8_t* __restrict__ codes_t = w.codes_t;
    uint32_t* __restrict__ stage = w.stage;
    int8_t* __restrict__ tgv = w.tgv;
    const Real* __restrict__ part = w.pst[w.cur];
    const int GGuP = w.GGuP;
    const int32_t* __restrict__ pof = w.pof;
    const Real* __restrict__ ptc = w.ptc;
    unsigned* __restrict__ cnt = w.cnt;
    const int16_t* __restrict__ irank = w.irank;
    const int32_t* __restrict__ prefix = w.prefix;
    const uint32_t seed = dM.seed;
    unsigned* __restrict__ amb = w.amb;
    for (int i = lane; i < N * 8; i += 32) cnt[i] = 0;
    for (int i = lane; i < w.S * 24; i += 32) amb[i] = 0;
    __syncwarp();
    int err = 0;
    const int rk = irank[w.root];
    unsigned n_tg = 0;
    // Emission histogram: once a node's base is drawn, the (base, parent base)
    // pair of its own branch and the (code, base) pairs of its leaf children
    // are counted (warp-aggregated with match-any; every non-root node of the
    // pruned tree is the child of exactly one internal node).
    auto hist = [&](int node, int key) {
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (key >= 0 && lane == __ffs(peers) - 1) {
            if (key < 16) {
                const int bin = node * 16 + key;
                atomicAdd(&cnt[bin >> 1], (unsigned)__popc(peers) << (16 * (bin & 1)));
            } else {
                atomicAdd(&amb[node * 24 + key - 16], (unsigned)__popc(peers));   // leaves only, rare
            }
        }
    };
    for (int g0 = 0; g0 < GG; g0 += 32 * C) {
        bool act[C];
        int pat[C];
#pragma unroll
        for (int j = 0; j < C; j++) {
            const int g = g0 + 32 * j + lane;
            act[j] = g < GG;
            pat[j] = act[j] ? pof[g] : 0;
            stage_column(codes_t, SP, stage + j * sstride, lane, g, act[j]);
        }
        auto leaf_pairs = [&](const NodeRec& R, int j, int base) {
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int c = q ? R.c1 : R.c0;
                if ((q ? R.r1 : R.r0) >= 0 || (q ? R.m1 : R.m0)) continue;
                int key = -1;
                if (act[j] && base < 4) {
                    const int code = stage_code(stage + j * sstride, c, lane);
                    const int sym = code < 4 ? code : (code >= CODE_R ? code - 2 : -1);
                    if (sym >= 0) key = sym * 4 + base;
                }
                hist(c, key);
            }
        };
        uint64_t wp[C], blk[C];
        uint32_t words[C][4];
        {
            const NodeRec RR = rec[rk];
#pragma unroll
            for (int j = 0; j < C; j++) {
                int nn = 4;
                if (act[j]) {
                    Real rootp[4];
                    ld4(part + ((size_t)rk * GGuP + pat[j]) * 4, rootp);
                    wp[j] = pos + (uint64_t)prefix[g0 + 32 * j + lane];
                    blk[j] = wp[j] >> 2;
                    philox4x32_10((uint32_t)blk[j], (uint32_t)(blk[j] >> 32), 0u, 0u, seed, 0u, words[j]);
                    nn = cat4(rootp, u_of<Real>(words[j][wp[j] & 3]));
                    wp[j]++;
                    if (nn > 3) { err = 1; nn = 0; }
                    tgv[(rk * C + j) * 32 + lane] = (int8_t)nn;
                    n_tg++;
                }
                leaf_pairs(RR, j, nn);
            }
        }
        // the partials of a node are read three nodes ahead: the loads are
        // gathers by pattern from L2 or HBM and their latency overlaps the
        // draws of the nodes in between
        Real cur[C][4], nx1[C][4], nx2[C][4], nx3[C][4];
        auto load_part = [&](Real (&dst)[C][4], int k) {
#pragma unroll
            for (int j = 0; j < C; j++) ld4(part + ((size_t)k * GGuP + pat[j]) * 4, dst[j]);
        };
        if (n_int >= 2) load_part(cur, n_int - 2);
        if (n_int >= 3) load_part(nx1, n_int - 3);
        if (n_int >= 4) load_part(nx2, n_int - 4);
        for (int k = n_int - 2; k >= 0; k--) {
            if (k >= 3) load_part(nx3, k - 3);
            const NodeRec R = rec[k];
#pragma unroll
            for (int j = 0; j < C; j++) {
                int n2 = 4, tp = 4;
                if (act[j]) {
                    int8_t* tk = tgv + (k * C + j) * 32 + lane;
                    if (R.missing || cur[j][0] < 0) {   // no data below the node (see column_up)
                        *tk = 4;
                    } else {
                        tp = tgv[(R.prank * C + j) * 32 + lane];
                        const Real* __restrict__ Ps = ptc + R.self * 16 + tp;
                        Real q[4];
#pragma unroll
                        for (int i = 0; i < 4; i++) q[i] = Ps[i * 4] * cur[j][i];
                        if ((wp[j] >> 2) != blk[j]) {
                            blk[j] = wp[j] >> 2;
                            philox4x32_10((uint32_t)blk[j], (uint32_t)(blk[j] >> 32), 0u, 0u, seed, 0u, words[j]);
                        }
                        n2 = cat4(q, u_of<Real>(words[j][wp[j] & 3]));
                        wp[j]++;
                        if (n2 > 3) { err = 1; n2 = 0; }
                        *tk = (int8_t)n2;
                        n_tg++;
                    }
                }
                hist(R.self, (n2 < 4 && tp < 4) ? n2 * 4 + tp : -1);
                leaf_pairs(R, j, n2);
            }
#pragma unroll
            for (int j = 0; j < C; j++)
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    cur[j][i] = nx1[j][i];
                    nx1[j][i] = nx2[j][i];
                    nx2[j][i] = nx3[j][i];
                }
        }
    }
    w.n_tg += n_tg;
    __syncwarp();
    return warp_or(err);
}

// Emission sums from the histogram (getEmission, bpp_c2.cpp:355-390).
template <typename Real, int C>
__device__ __noinline__ void emission_sums(W<Real, C>& w) {
    const int NB = NSYM * 4;
    for (int t = w.lane; t < (w.n_nodes - 1) * 3; t += 32) {
        int s = w.nodes[t / 3];
        int z = t % 3;
        if (w.missing[s]) continue;
        const double* P = w.tbl + ((size_t)z * w.N + s) * 16;
        double e = 0;
        // bins 0..15 are packed pairs in shared memory; only leaves can carry
        // ambiguity codes (bins 16..39, device memory)
        const int nb = s >= w.S ? 16 : NB;
        for (int b = 0; b < nb; b++) {
            unsigned n;
            if (b < 16) {
                const unsigned word = w.cnt[(s * 16 + b) >> 1];
                if (!word) { b |= 1; continue; }   // both bins of the pair are empty
                n = (word >> (16 * (b & 1))) & 0xFFFF;
            } else {
                n = w.amb[s * 24 + b - 16];
            }
            if (!n) continue;
            int sym = b >> 2, tp = b & 3;
            double v;
            if (sym < 4) {
                v = (sizeof(Real) == 8) ? d_log(P[sym * 4 + tp]) : (double)f_log((float)P[sym * 4 + tp]);
            } else {
                int msk = ambig_mask(sym - 4);
                double tt = 0;
                for (int q = 0; q < 4; q++)
                    if (msk & (1 << q)) tt += P[q * 4 + tp];
                v = (sizeof(Real) == 8) ? d_log(tt) : (double)f_log((float)tt);
            }
            e += (double)n * v;
        }
        w.emis[s * 3 + z] = e;
    }
    wsync();
}

// Latent-state forward filter (linear FP64, normalised per node) and
// backward sampling (Update_Z_subtree, bpp_c.cpp:1182-1293).
template <typename Real, int C>
__device__ __noinline__ int update_z(W<Real, C>& w, uint64_t pos) {
    // transition T[zc][zp] for fixed (fixZ) and free nodes from g, l, l2 (bpp_c.cpp:573-599)
    const double gr = w.st.gr, lr = w.st.lr, lr2 = w.st.lr2;
    double Tf[3][3] = {{1 - gr, 0, 0}, {gr, 1, 0}, {0, 0, 0}};
    double Tn[3][3] = {{1 - gr, 0, 0}, {gr, 1 - lr, lr2}, {0, lr, 1 - lr2}};
    // node beta := exp(emission - max) with state 2 banned for fixZ nodes
    for (int i = w.lane; i < w.n_nodes; i += 32) {
        int s = w.nodes[i];
        double e0 = w.emis[s * 3 + 0], e1 = w.emis[s * 3 + 1], e2 = w.emis[s * 3 + 2];
        bool ban = w.fixZ[s] == 1;
        double mx = e0 > e1 ? e0 : e1;
        if (!ban && e2 > mx) mx = e2;
        w.bz[s * 3 + 0] = d_exp(e0 - mx);
        w.bz[s * 3 + 1] = d_exp(e1 - mx);
        w.bz[s * 3 + 2] = ban ? 0.0 : d_exp(e2 - mx);
    }
    wsync();
    for (int h = 0; h < w.n_hlev; h++) {
        int a = w.hlev_start[h], b = w.hlev_start[h + 1];
        for (int i = a + w.lane; i < b; i += 32) {
            int p = w.hlev_nodes[i];
            double v[3] = {w.bz[p * 3 + 0], w.bz[p * 3 + 1], w.bz[p * 3 + 2]};
            int ch[2] = {w.c2a[p], w.c2b[p]};
            for (int q = 0; q < 2; q++) {
                int c = ch[q];
                const double(*T)[3] = (w.fixZ[c] == 1) ? Tf : Tn;
                for (int zp = 0; zp < 3; zp++) {
                    double m = 0;
                    for (int zc = 0; zc < 3; zc++) m += T[zc][zp] * w.bz[c * 3 + zc];
                    v[zp] *= m;
                }
            }
            double mx = fmax(v[0], fmax(v[1], v[2]));
            double inv = mx > 0 ? 1.0 / mx : 1.0;
            for (int zp = 0; zp < 3; zp++) w.bz[p * 3 + zp] = v[zp] * inv;
        }
        wsync();
    }
    int err = 0;
    if (w.lane == 0) {
        double pr[3] = {0.5 * w.bz[w.root * 3 + 0], 0.5 * w.bz[w.root * 3 + 1], 0.0};
        uint32_t wd[4];
        philox4x32_10((uint32_t)(pos >> 2), (uint32_t)(pos >> 34), 0u, 0u, dM.seed, 0u, wd);
        int nn = categorical(3, pr, word_to_uniform(wd[pos & 3]));
        if (nn > 2) { err = 1; nn = w.Z[w.root]; }
        w.chg[w.root] = (nn != w.Z[w.root]);
        w.Z[w.root] = (int8_t)nn;
    }
    wsync();
    for (int d = 0; d < w.n_dlev; d++) {
        int a = w.dlev_start[d], b = w.dlev_start[d + 1];
        for (int i = a + w.lane; i < b; i += 32) {
            int s = w.dlev_nodes[i];
            int zp = w.Z[w.par[s]];
            const double(*T)[3] = (w.fixZ[s] == 1) ? Tf : Tn;
            double pr[3];
            for (int k = 0; k < 3; k++) pr[k] = T[k][zp] * w.bz[s * 3 + k];
            uint64_t wq = pos + 1 + (uint64_t)(w.n_nodes - 2 - w.pos[s]);
            uint32_t wd[4];
            philox4x32_10((uint32_t)(wq >> 2), (uint32_t)(wq >> 34), 0u, 0u, dM.seed, 0u, wd);
            int nn = categorical(3, pr, word_to_uniform(wd[wq & 3]));
            if (nn > 2) { err = 1; nn = w.Z[s]; }
            w.chg[s] = (nn != w.Z[s]);
            w.Z[s] = (int8_t)nn;
        }
        wsync();
    }
    return warp_or(err);
}

// Flags of proper ancestors (getUpdateNode, bpp_c.cpp:620-642, 836-858).
// mode 0: of changed nodes; 1: of non-missing Z == 2; 2: of non-missing Z == 1.
template <typename Real, int C>
__device__ __noinline__ int ancestors(W<Real, C>& w, int mode, int8_t* dst) {
    for (int i = w.lane; i < w.N; i += 32) dst[i] = 0;
    wsync();
#pragma unroll 1
    for (int i = w.lane; i < w.n_nodes; i += 32) {
        int s = w.nodes[i];
        bool f = (mode == 0) ? (w.chg[s] != 0) : (!w.missing[s] && w.Z[s] == (mode == 1 ? 2 : 1));
        if (!f) continue;
        int j = w.par[s];
#pragma unroll 1
        while (j >= 0 && j < w.N) {
            dst[j] = 1;
            j = w.par[j];
        }
    }
    wsync();
    return dst[w.root];
}

__device__ __forceinline__ double bcast(double v) { return __shfl_sync(0xffffffffu, v, 0); }
__device__ __forceinline__ int bcast(int v) { return __shfl_sync(0xffffffffu, v, 0); }
__device__ __forceinline__ uint64_t bcast(uint64_t v) {
    return ((uint64_t)__shfl_sync(0xffffffffu, (unsigned)(v >> 32), 0) << 32) | __shfl_sync(0xffffffffu, (unsigned)v, 0);
}

// One MH update of the accelerated (neut) or conserved rate (sample_rate,
// bpp_c.cpp:930-1176; M = 1, adaptive factor 0.5).  Lane 0 draws and decides,
// the warp evaluates the proposal's likelihood.
template <typename Real, int C>
__device__ __noinline__ double mh_rate(W<Real, C>& w, bool neut, double old_rate, int m) {
    const double prior_a = neut ? dM.nprior_a : dM.cprior_a;
    const double prior_b = neut ? dM.nprior_b : dM.cprior_b;
    const int cls = neut ? C_NEUT : C_CONS;
    const int resZ = w.st.resZ;
    int any = ancestors(w, neut ? 1 : 2, w.unv);
    double cur = old_rate;
    if (!any) {
        // no branch of the class: draw from the prior (bpp_c.cpp:940-964)
        double c0 = old_rate;
        uint64_t pos = w.st.pos;
        if (w.lane == 0 && resZ != 0) {
            StreamReader rd;
            rd.init(dM.seed, pos);
            c0 = rd.gamma(prior_a, prior_b);
            pos = rd.pos;
            if (neut) {
                if (dM.ropt == 1 && c0 < dM.nlb) c0 = old_rate;
                else if (dM.ropt == 2 && c0 < w.trd[TR_C * w.T + m]) c0 = old_rate;
            } else {
                if (dM.ropt == 1 && c0 > dM.cub) c0 = old_rate;
                else if (dM.ropt == 2 && c0 > w.trd[TR_N * w.T + m + 1]) c0 = old_rate;
            }
        }
        cur = bcast(c0);
        w.st.pos = bcast(pos);
        if (cur != old_rate) build_table(w, cls, cur, true, false, true);
    } else {
        double r = 0, proposal = 0;
        int skip = 0;
        uint64_t pos = w.st.pos;
        if (w.lane == 0) {
            StreamReader rd;
            rd.init(dM.seed, pos);
            r = rd.uniform();
            if (neut) {
                proposal = rd.gamma(__ddiv_rn(old_rate, w.st.prop_n), w.st.prop_n);
                if (dM.ropt == 1 && proposal < dM.nlb) skip = 1;
                else if (dM.ropt == 2 && proposal < w.trd[TR_C * w.T + m]) skip = 1;
            } else {
                double ip = __ddiv_rn(1.0, w.st.prop_c);
                double u = __dadd_rn(__dmul_rn(r, __dsub_rn(w.st.prop_c, ip)), ip);
                proposal = __dmul_rn(old_rate, u);
                if (dM.ropt == 1 && proposal > dM.cub) skip = 1;
                else if (dM.ropt == 2 && proposal > w.trd[TR_N * w.T + m + 1]) skip = 1;
            }
            if (!skip && (proposal < 1e-12 || proposal > 1e8)) skip = 1;
            pos = rd.pos;
        }
        skip = bcast(skip);
        proposal = bcast(proposal);
        w.st.pos = bcast(pos);
        if (!skip) {
            fill_ptc(w, cls, proposal);
            double ll_new = likelihood_pass(w, w.cur ^ 1);   // proposal partials into the other buffer
            int acc = 0;
            if (w.lane == 0) {
                double MH;
                if (neut)
                    MH = __dsub_rn(__dadd_rn(__dsub_rn(__dadd_rn(__dsub_rn(ll_new, w.st.loglik),
                                                               log_gamma_pdf(proposal, prior_a, prior_b)),
                                                     log_gamma_pdf(old_rate, prior_a, prior_b)),
                                           log_gamma_pdf(old_rate, __ddiv_rn(proposal, w.st.prop_n), w.st.prop_n)),
                                   log_gamma_pdf(proposal, __ddiv_rn(old_rate, w.st.prop_n), w.st.prop_n));
                else
                    MH = __dsub_rn(__dadd_rn(__dsub_rn(__dadd_rn(__dsub_rn(ll_new, w.st.loglik),
                                                               log_gamma_pdf(proposal, prior_a, prior_b)),
                                                     log_gamma_pdf(old_rate, prior_a, prior_b)),
                                           d_log(old_rate)),
                                   d_log(proposal));
                acc = d_log(r) < MH;
            }
            acc = bcast(acc);
            if (acc) {
                cur = proposal;
                w.st.loglik = ll_new;
                w.cur ^= 1;   // the proposal's partials become the current ones
                build_table(w, cls, cur, true, false, true);
            }
        }
    }
    if (cur != old_rate) { if (neut) w.st.acc_n++; else w.st.acc_c++; }
    // adaptive proposal scale (bpp_c.cpp:1145-1171); every lane computes the same values
    if ((m + 1) % dM.adapt_freq == 0) {
        int blocks = (m + 1) / dM.adapt_freq;
        double step = fmin(0.5, 1 / sqrt((double)blocks));
        double scale_adj;
        if (neut) {
            double rate = (double)w.st.acc_n / dM.adapt_freq;
            scale_adj = rate > 0.44 ? d_exp(step) : (rate < 0.23 ? d_exp(-step) : 1.0);
            w.st.prop_n = __dmul_rn(w.st.prop_n, scale_adj);
            if (w.st.prop_n > 1) w.st.prop_n = 1;
            w.st.acc_n = 0;
        } else {
            double rate = (double)w.st.acc_c / dM.adapt_freq;
            scale_adj = rate > 0.44 ? d_exp(step) : (rate < 0.23 ? d_exp(-step) : 1.0);
            w.st.prop_c = d_pow(w.st.prop_c, scale_adj);
            if (w.st.prop_c < 1.0001) w.st.prop_c = 1.0001;
            w.st.acc_c = 0;
        }
    }
    return cur;
}

// Prior of a Z configuration (bpp_c2.cpp:131-163).
template <typename Real, int C>
__device__ __noinline__ double prior_config(W<Real, C>& w, const int8_t* z) {
    double nZ[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int k = 0; k + 1 < w.n_nodes; k++) {
        int s = w.nodes[k];
        nZ[z[s]][z[w.par[s]]] += 1;
    }
    double pz = lnbeta(dM.ga + nZ[1][0] + nZ[2][0], dM.gb + nZ[0][0]) - lnbeta(dM.ga, dM.gb);
    for (int k = 0; k + 1 < w.n_nodes; k++) {
        int s = w.nodes[k];
        if (w.fixZ[s] == 1) nZ[z[s]][z[w.par[s]]] -= 1;
    }
    pz += lnbeta(dM.la + nZ[2][1], dM.lb + nZ[1][1]) - lnbeta(dM.la, dM.lb);
    if (dM.l2a > 0) pz += lnbeta(dM.l2a + nZ[1][2], dM.l2b + nZ[2][2]) - lnbeta(dM.l2a, dM.l2b);
    pz += (z[w.root] == 2) ? -CUDART_INF : d_log(0.5);
    return pz;
}

// Marginal likelihood of one model (Eval2, bpp_c2.cpp:14-353) by one warp.
template <typename Real, int C>
__device__ __noinline__ double eval2(W<Real, C>& w, char* gws, int* n_conf_out) {
    const int burn = w.burn, mcmc = w.mcmc, T = w.T, N = w.N;
    const int resZ = w.st.resZ;
    GrpLayout G = GrpLayout::make(mcmc, w.n_int_max, sizeof(Real), w.GGuP, N);
    uint64_t* hash = (uint64_t*)(gws + G.hash);
    int32_t* rep = (int32_t*)(gws + G.rep);
    int32_t* cfg = (int32_t*)(gws + G.cfg);
    int32_t* nxt = (int32_t*)(gws + G.nxt);
    int32_t* head = (int32_t*)(gws + G.head);
    int32_t* first = (int32_t*)(gws + G.first);
    double* CNT = (double*)(gws + G.cstat);
    double* VC = CNT + (mcmc + 2);
    double* MC = VC + (mcmc + 2);
    double* VN = MC + (mcmc + 2);
    double* MN = VN + (mcmc + 2);
    double* CV = MN + (mcmc + 2);
    double* SF = CV + (mcmc + 2);
    double* LD = SF + (mcmc + 2);
    const int8_t* Zm = w.smaxz;
    int8_t* unc = w.mask;
    for (int s = w.lane; s < N; s += 32) {
        int c = 0;
        for (int i = burn; i < T; i++) c += (w.trz[(size_t)i * N + s] == Zm[s]);
        unc[s] = c < mcmc;
    }
    wsync();
    for (int i = burn + w.lane; i <= T; i += 32) {
        const int8_t* z = (i < T) ? w.trz + (size_t)i * N : Zm;
        uint64_t h = 0xcbf29ce484222325ull;
        for (int s = 0; s < N; s++)
            if (unc[s]) h = fnv_step(h, (uint8_t)z[s]);
        hash[i - burn] = h;
    }
    wsync();
    auto same = [&](const int8_t* a, const int8_t* b) {
        for (int s = 0; s < N; s++)
            if (unc[s] && a[s] != b[s]) return false;
        return true;
    };
    for (int i = burn + w.lane; i < T; i += 32) {
        const int8_t* zi = w.trz + (size_t)i * N;
        uint64_t hi = hash[i - burn];
        int r = i;
        for (int j = T - 1; j > i; j--)
            if (hash[j - burn] == hi && same(w.trz + (size_t)j * N, zi)) { r = j; break; }
        rep[i - burn] = r;
        cfg[i - burn] = (hi == hash[T - burn] && same(zi, Zm)) ? -2 : -1;
    }
    wsync();
    int nconf = 1;
    if (w.lane == 0) {
        first[0] = -1;
        for (int i = T - 1; i >= burn; i--) {
            int k = i - burn;
            int j;
            if (cfg[k] == -2) j = 0;
            else if (rep[k] == i) { j = nconf++; first[j] = i; }
            else j = cfg[rep[k] - burn];
            cfg[k] = j;
        }
        for (int j = 0; j < nconf; j++) head[j] = -1;
        for (int i = burn; i < T; i++) {
            int k = i - burn;
            nxt[k] = head[cfg[k]];
            head[cfg[k]] = k;
        }
    }
    nconf = bcast(nconf);
    __syncwarp();
    *n_conf_out = nconf;
    const double* trN = w.trd + TR_N * T;
    const double* trC = w.trd + TR_C * T;
    const double* trF = w.trd + TR_FULL * T;
    for (int j = w.lane; j < nconf; j += 32) {
        double n = 0, vc = 0, mc = 0, vn = 0, mn = 0, cv = 0, sf = 0;
        for (int k = head[j]; k >= 0; k = nxt[k]) {
            int i = k + burn;
            n += 1;
            vc = __dadd_rn(vc, __dmul_rn(trC[i], trC[i]));
            mc = __dadd_rn(mc, trC[i]);
            if (resZ != 0) {
                vn = __dadd_rn(vn, __dmul_rn(trN[i], trN[i]));
                mn = __dadd_rn(mn, trN[i]);
                cv = __dadd_rn(cv, __dmul_rn(trC[i], trN[i]));
            }
            sf = __dadd_rn(sf, __ddiv_rn(trF[i], (double)mcmc));
        }
        CNT[j] = n; VC[j] = vc; MC[j] = mc; VN[j] = vn; MN[j] = mn; CV[j] = cv; SF[j] = sf;
        LD[j] = 0;
        double wgt = n / mcmc;
        if (wgt < 0.02) continue;
        const int8_t* z = (j == 0) ? Zm : w.trz + (size_t)first[j] * N;
        double pz = prior_config(w, z);
        SF[j] = __dadd_rn(SF[j], __ddiv_rn(__dmul_rn(n, pz), (double)mcmc));
        double ld;
        if (resZ == 0) {
            ld = __dsub_rn(d_log(__dsub_rn(vc, __ddiv_rn(__dmul_rn(mc, mc), n))), d_log(n));
        } else {
            double a = __dsub_rn(vc, __ddiv_rn(__dmul_rn(mc, mc), n));
            double b = __dsub_rn(vn, __ddiv_rn(__dmul_rn(mn, mn), n));
            double cov = __dsub_rn(cv, __ddiv_rn(__dmul_rn(mn, mc), n));
            ld = __dsub_rn(d_log(__dsub_rn(__dmul_rn(a, b), __dmul_rn(cov, cov))), __dmul_rn(2.0, d_log(n)));
        }
        LD[j] = ld;
    }
    __syncwarp();
    double VB = 0;
    int eff = 0;
    if (w.lane == 0) {
        for (int j = 0; j < nconf; j++) {
            double wgt = CNT[j] / mcmc;
            if (wgt < 0.02) continue;
            if (isnan(LD[j])) continue;
            eff += (int)CNT[j];
            VB = __dsub_rn(VB, __dmul_rn(wgt, d_log(CNT[j])));
            VB = __dadd_rn(VB, SF[j]);
            VB = __dadd_rn(VB, __ddiv_rn(__dmul_rn(__dmul_rn(0.5, LD[j]), CNT[j]), (double)mcmc));
        }
    }
    eff = bcast(eff);
    VB = bcast(VB);
    if (eff == 0) {
        // fallback: prune each configuration at the mean rates (bpp_c2.cpp:199-316)
        double varn = 0, varc = 0, cov = 0, meann = 0, meanc = 0;
        for (int j = 0; j < nconf; j++) {
            varc = __dadd_rn(varc, VC[j]);
            meanc = __dadd_rn(meanc, MC[j]);
            if (resZ != 0) { meann = __dadd_rn(meann, MN[j]); varn = __dadd_rn(varn, VN[j]); cov = __dadd_rn(cov, CV[j]); }
        }
        double rn = meann / mcmc, rc = meanc / mcmc;
        build_table(w, C_CONS, rc, true, true, false);
        if (resZ != 0) build_table(w, C_NEUT, rn, true, true, false);
        for (int j = 0; j < nconf; j++) {
            const int8_t* z = (j == 0) ? Zm : w.trz + (size_t)first[j] * N;
            for (int s = w.lane; s < N; s += 32) w.Z[s] = z[s];
            wsync();
            double pz = prior_config(w, z);
            fill_ptc(w, -1, 0.0);
            double ll = likelihood_pass(w, w.cur ^ 1);   // the chain is over: either buffer may be overwritten
            if (w.lane == 0) SF[j] = __dadd_rn(ll, pz);
        }
        __syncwarp();
        double v = 0;
        if (w.lane == 0) {
            double mx = SF[0];
            for (int j = 1; j < nconf; j++) if (SF[j] > mx) mx = SF[j];
            if (mx == -CUDART_INF) v = -CUDART_INF;
            else {
                double sm = 0;
                for (int j = 0; j < nconf; j++) sm = __dadd_rn(sm, d_exp(__dsub_rn(SF[j], mx)));
                v = __dadd_rn(d_log(sm), mx);
            }
            v = __dadd_rn(v, log_gamma_pdf(rc, dM.cprior_a, dM.cprior_b));
            if (resZ != 0) v = __dadd_rn(v, log_gamma_pdf(rn, dM.nprior_a, dM.nprior_b));
            double logdet;
            if (resZ == 0) {
                varc = __dsub_rn(varc, __ddiv_rn(__dmul_rn(meanc, meanc), (double)mcmc));
                logdet = __dsub_rn(d_log(varc), d_log((double)mcmc));
                v = __dadd_rn(v, __dadd_rn(__dmul_rn(0.5, logdet), __dmul_rn(0.5, d_log(2 * CUDART_PI))));
            } else {
                varn = __dsub_rn(varn, __ddiv_rn(__dmul_rn(meann, meann), (double)mcmc));
                varc = __dsub_rn(varc, __ddiv_rn(__dmul_rn(meanc, meanc), (double)mcmc));
                cov = __dsub_rn(cov, __ddiv_rn(__dmul_rn(meann, meanc), (double)mcmc));
                logdet = __dsub_rn(d_log(__dsub_rn(__dmul_rn(varc, varn), __dmul_rn(cov, cov))),
                                   __dmul_rn(2.0, d_log((double)mcmc)));
                v = __dadd_rn(v, __dadd_rn(__dmul_rn(0.5, logdet), d_log(2 * CUDART_PI)));
            }
        }
        VB = bcast(v);
    } else {
        double f = (double)mcmc / eff;
        if (resZ != 0) VB = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(VB, f), d_log((double)mcmc)), d_log(2 * CUDART_PI)), 1.0);
        else VB = __dadd_rn(__dadd_rn(__dmul_rn(VB, f), d_log((double)mcmc)), __dmul_rn(0.5, __dadd_rn(d_log(2 * CUDART_PI), 1.0)));
    }
    return VB;
}

// Element of rank T/2 under std::sort's order (bpp_c2.cpp:742-755).
__device__ __noinline__ double warp_median(const double* x, int T) {
    int target = T / 2;
    double found = 0;
    int hit = 0;
    for (int i = threadIdx.x & 31; i < T; i += 32) {
        double v = x[i];
        int r = 0;
        for (int j = 0; j < T; j++) {
            double u = x[j];
            r += (u < v) || (u == v && j < i);
        }
        if (r == target) { found = v; hit = 1; }
    }
    unsigned b = __ballot_sync(0xffffffffu, hit);
    return __shfl_sync(0xffffffffu, found, __ffs(b) - 1);
}

// initMCMC for model w.st.mi (bpp_c.cpp:131-343) followed by the initial full prune.
template <typename Real, int C>
__device__ __noinline__ void init_model(W<Real, C>& w) {
    const int resZ = w.st.resZ;
    for (int i = w.lane; i < w.N; i += 32) { w.Z[i] = -1; w.fixZ[i] = -1; }
    wsync();
    for (int i = w.lane; i < w.n_nodes; i += 32) {
        int s = w.nodes[i];
        w.Z[s] = (s == w.root) ? 0 : 1;
        if (w.upc[s] || s == w.root) w.fixZ[s] = 1;
        if (resZ == 2 && w.upcc[s]) w.fixZ[s] = 1;
        if (resZ == 0 && s != w.root) w.fixZ[s] = 1;
    }
    wsync();
    w.st.prop_c = 1.2;
    w.st.prop_n = (double)1 / w.GG * 10;
    w.st.maxll = -CUDART_INF;
    w.st.max_m = 0;
    w.st.m = 0;
    w.st.rate_n = dM.init_n;
    w.st.rate_c = dM.init_c;
    w.st.gr = dM.init_g;
    w.st.lr = dM.init_l;
    w.st.lr2 = (dM.l2a == 0) ? 0.0 : dM.init_l2;
    if (w.lane == 0) {
        w.trd[TR_N * w.T] = w.st.rate_n;
        w.trd[TR_C * w.T] = w.st.rate_c;
        w.trd[TR_G * w.T] = w.st.gr;
        w.trd[TR_L * w.T] = w.st.lr;
        w.trd[TR_L2 * w.T] = w.st.lr2;
    }
    build_table(w, C_NULL, 1.0, false, false, false);
    build_table(w, C_NEUT, dM.init_n, true, false, false);
    build_table(w, C_CONS, dM.init_c, true, false, false);
    fill_ptc(w, -1, 0.0);
    w.cur = 0;
    w.st.loglik = likelihood_pass(w, w.cur);
    w.st.phase = PH_RUN;
}

template <typename Real, int C>
__device__ __noinline__ void write_slot_z(W<Real, C>& w) {
    for (int i = w.lane; i < w.N; i += 32) w.sZ[i] = w.Z[i];
}

// ---------------------------------------------------------------------------
// kernel
// ---------------------------------------------------------------------------
template <typename Real, int C>
__global__ void __launch_bounds__(128) batch_kernel(BatchParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int N = dM.N, S = dM.S;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    WarpSmem<Real> L = WarpSmem<Real>::make(N, P.n_int_max, S, P.stack_depth, C);
    TopoLayout TL = TopoLayout::make(N);
    unsigned char* base = smem + (size_t)wid * L.total;
    W<Real, C> w;
    w.lane = lane;
    w.S = S;
    w.N = N;
    w.burn = dM.burnin;
    w.mcmc = dM.mcmc;
    w.T = dM.burnin + dM.mcmc;
    w.ptc = (Real*)(base + L.ptc);
    w.part = (Real*)(base + L.part);
    w.emis = (double*)(base + L.part);
    w.bz = w.emis + (size_t)N * 3;
    w.tgv = (int8_t*)(base + L.tgv);
    int16_t* t16 = (int16_t*)(base + L.topo);
    w.nodes = t16 + TL.nodes; w.internal = t16 + TL.internal; w.c2a = t16 + TL.c2a; w.c2b = t16 + TL.c2b;
    w.par = t16 + TL.par; w.irank = t16 + TL.irank; w.pos = t16 + TL.pos; w.missing = t16 + TL.missing;
    w.upc = t16 + TL.upc; w.upcc = t16 + TL.upcc; w.hlev_start = t16 + TL.hlev_start;
    w.hlev_nodes = t16 + TL.hlev_nodes; w.dlev_start = t16 + TL.dlev_start; w.dlev_nodes = t16 + TL.dlev_nodes;
    w.dist2 = (double*)(base + L.dbl);
    NodeRec* recw = (NodeRec*)(base + L.rec);
    w.rec = recw;
    NodeRec* srecw = (NodeRec*)(base + L.srec);
    w.srec = srecw;
    w.stage = (uint32_t*)(base + L.stage);
    w.cnt = (unsigned*)(base + L.cnt);
    int8_t* f8 = (int8_t*)(base + L.i8);
    w.fixZ = f8; w.chg = f8 + N; w.unv = f8 + 2 * N; w.mask = f8 + 3 * N; w.Z = f8 + 5 * N;
    const int gw = blockIdx.x * nw + wid;
    const int n_gw = gridDim.x * nw;
    char* gws = P.grp_ws + (size_t)gw * P.grp_ws_stride;
    {
        GrpLayout GLy = GrpLayout::make(dM.mcmc, P.n_int_max, sizeof(Real), P.GGuP_max, N);
        w.pst[0] = (Real*)(gws + GLy.pst);
        w.pst[1] = w.pst[0] + (size_t)P.n_int_max * P.GGuP_max * 4;
        w.GGuP = P.GGuP_max;
        w.n_int_max = P.n_int_max;
        w.amb = (unsigned*)(gws + GLy.amb);
    }
    const SlotLayout SL = SlotLayout::make(N, w.T);
    const int TI = dM.trace_iters < w.T ? dM.trace_iters : w.T;
    const int resZ_of[3] = {0, 2, 1};
    (void)n_gw;
    for (;;) {
        int slot = 0;
        if (lane == 0) slot = atomicAdd(P.next_slot, 1);
        slot = __shfl_sync(0xffffffffu, slot, 0);
        if (slot >= P.n_slots) break;
        SlotState* sp = P.slots + slot;
        w.st = *sp;
        if (w.st.phase == PH_DONE || w.st.phase == PH_EMPTY || w.st.elem < 0) continue;
        const int e = w.st.elem;
        const ElemHeader& H = P.hdr[e];
        w.GG = H.GG; w.GGp = H.GGp; w.root = H.root; w.n_nodes = H.n_nodes; w.n_int = H.n_int;
        w.n_hlev = H.n_hlev; w.n_dlev = H.n_dlev; w.tg_draws = H.tg_draws;
        w.codes = P.blob + H.codes_off;
        w.codes_t = P.blob + H.codes_t_off;
        w.pof = (const int32_t*)(P.blob + H.pof_off);
        w.cur = 0;
        w.pcodes_t = P.blob + H.pcodes_off;
        w.pw = (const int32_t*)(P.blob + H.pw_off);
        w.GGu = H.GGu;
        w.SP = H.SP;
        w.prefix = (const int32_t*)(P.blob + H.prefix_off);
        {
            const int16_t* topo = (const int16_t*)(P.blob + H.topo_off);
            for (int i = lane; i < TL.total; i += 32) t16[i] = topo[i];
            const double* d2 = (const double*)(P.blob + H.topo_off + (size_t)((TL.total * 2 + 15) & ~15));
            for (int i = lane; i < N; i += 32) w.dist2[i] = d2[i];
        }
        wsync();
        for (int k = lane; k < w.n_int; k += 32) {
            int s = w.internal[k];
            NodeRec R;
            R.c0 = w.c2a[s];
            R.c1 = w.c2b[s];
            R.r0 = R.c0 >= S ? w.irank[R.c0] : -1;
            R.r1 = R.c1 >= S ? w.irank[R.c1] : -1;
            R.m0 = (int8_t)w.missing[R.c0];
            R.m1 = (int8_t)w.missing[R.c1];
            R.missing = (int8_t)w.missing[s];
            R.is_root = (s == w.root);
            R.self = (int16_t)s;
            R.prank = (s == w.root) ? (int16_t)-1 : w.irank[w.par[s]];
            recw[k] = R;
        }
        {
            const int16_t* sord = t16 + TL.sord;
            const int16_t* sflag = t16 + TL.sflag;
            for (int k = lane; k < w.n_int; k += 32) {
                int s = sord[k];
                NodeRec R;
                R.c0 = w.c2a[s];
                R.c1 = w.c2b[s];
                R.r0 = R.c0 >= S ? w.irank[R.c0] : -1;
                R.r1 = R.c1 >= S ? w.irank[R.c1] : -1;
                R.m0 = (int8_t)w.missing[R.c0];
                R.m1 = (int8_t)w.missing[R.c1];
                R.missing = (int8_t)w.missing[s];
                R.is_root = (s == w.root);
                R.self = w.irank[s];      // stack order: self = internal rank (scratch row)
                R.prank = sflag[s];       // stack order: bit 0 = first child's partial on top
                srecw[k] = R;
            }
        }
        char* sw = P.slot_ws + (size_t)slot * P.slot_ws_stride;
        w.sZ = (int8_t*)(sw + SL.Z);
        w.smaxz = (int8_t*)(sw + SL.maxz);
        w.tbl = (double*)(sw + SL.tbl);
        w.trz = (int8_t*)(sw + SL.trz);
        w.trd = (double*)(sw + SL.trd);
        w.e_int = w.e_leaf = w.n_tg = 0;
        for (int q = 0; q < 8; q++) w.ph[q] = 0;
        w.t0 = clock64();
        if (w.st.phase == PH_INIT && w.st.mi == 0 && lane == 0) w.st.start_clock = clock64();
        // restore Z / fixZ of a running model
        if (w.st.phase == PH_RUN) {
            for (int i = lane; i < N; i += 32) { w.Z[i] = w.sZ[i]; w.fixZ[i] = -1; }
            wsync();
            const int resZ = w.st.resZ;
            for (int i = lane; i < w.n_nodes; i += 32) {
                int s = w.nodes[i];
                if (w.upc[s] || s == w.root) w.fixZ[s] = 1;
                if (resZ == 2 && w.upcc[s]) w.fixZ[s] = 1;
                if (resZ == 0 && s != w.root) w.fixZ[s] = 1;
            }
            wsync();
            // the partial buffers belong to the warp, not the slot: rebuild the
            // current state's partials (the log-likelihood itself is kept)
            fill_ptc(w, -1, 0.0);
            likelihood_pass(w, w.cur);
        }
        wsync();
        // iterations this launch: `sweeps` for a 256-column element, scaled by
        // 256 / GG so that every chain's share of a launch costs about the same
        int budget = 0x7fffffff;
        if (P.sweeps > 0) {
            long long b = (long long)P.sweeps * 256 / (w.GG > 0 ? w.GG : 1);
            budget = (int)(b < 1 ? 1 : (b > 0x7fffffff ? 0x7fffffff : b));
        }
        int errs = 0;
        while (budget > 0 && w.st.phase != PH_DONE) {
            if (w.st.phase == PH_INIT) {
                w.st.resZ = resZ_of[w.st.mi];
                init_model(w);
                PHASE(7);
            }
            const int m = w.st.m;
            const int T = w.T;
            // MonitorChain (bpp_c.cpp:741-834)
            for (int i = lane; i < N; i += 32) w.trz[(size_t)m * N + i] = w.Z[i];
            double full = w.st.loglik + 0.0;
            full += log_gamma_pdf(w.trd[TR_C * T + m], dM.cprior_a, dM.cprior_b);
            if (w.st.resZ != 0) full += log_gamma_pdf(w.trd[TR_N * T + m], dM.nprior_a, dM.nprior_b);
            if (lane == 0) { w.trd[TR_LL * T + m] = w.st.loglik; w.trd[TR_FULL * T + m] = full; }
            if (m >= w.burn && full > w.st.maxll) {
                w.st.maxll = full;
                w.st.max_m = m;
                for (int i = lane; i < N; i += 32) w.smaxz[i] = w.Z[i];
            }
            wsync();
            if (m == T - 1) {
                // end of the model: Eval2 and the output row (bpp_c2.cpp:14-353, 739-785)
                const int mi = w.st.mi;
                DevModelResult& MR = P.results[e].model[mi];
                if (TI > 0 && P.tr_d) {
                    double* td = P.tr_d + ((size_t)e * 3 + mi) * 6 * TI;
                    const int rows[6] = {TR_LL, TR_N, TR_C, TR_G, TR_L, TR_L2};
                    for (int i = lane; i < 6 * TI; i += 32) td[i] = w.trd[rows[i / TI] * T + (i % TI)];
                    int8_t* tz = P.tr_z + ((size_t)e * 3 + mi) * TI * N;
                    for (int i = lane; i < TI * N; i += 32) tz[i] = w.trz[i];
                }
                __syncwarp();
                int nconf = 0;
                double vb = eval2(w, gws, &nconf);
                const int mrow[5] = {TR_N, TR_C, TR_G, TR_L, TR_L2};
                double med[5];
                for (int q = 0; q < 5; q++) med[q] = warp_median(w.trd + mrow[q] * T, T);
                if (lane == 0) {
                    MR.loglik = vb;
                    MR.max_loglik = w.st.maxll;
                    for (int q = 0; q < 5; q++) MR.rates[q] = med[q];
                    MR.failure = isnan(vb) ? 1 : 0;
                    MR.n_configs = nconf;
                }
                if (isnan(vb)) w.st.status |= 2;
                int32_t* mz = P.max_z + ((size_t)e * 3 + mi) * N;
                for (int s = lane; s < N; s += 32) mz[s] = w.smaxz[s];
                double* pz = P.post_z + ((size_t)e * 3 + mi) * N * 4;
                for (int s = lane; s < N; s += 32) {
                    int c4[4] = {0, 0, 0, 0};
                    for (int i = w.burn; i < T; i++) {
                        int z = w.trz[(size_t)i * N + s];
                        if (z >= -1 && z <= 2) c4[z + 1]++;
                    }
                    if (w.missing[s]) c4[0] = w.mcmc;
                    for (int k = 0; k < 4; k++) pz[s * 4 + k] = (double)c4[k] / w.mcmc;
                }
                PHASE(7);
                w.st.mi++;
                w.st.phase = (w.st.mi == 3) ? PH_DONE : PH_INIT;
                if (w.st.phase == PH_DONE && lane == 0) {
                    P.results[e].status = (w.st.status & 1) ? 3 : ((w.st.status & 2) ? 2 : 0);
                    P.results[e].device_ms = (double)(clock64() - w.st.start_clock);
                    int di = atomicAdd(P.n_done, 1);
                    if (P.done_list) P.done_list[di] = slot;
                }
                __syncwarp();
                continue;
            }
            PHASE(6);
            // internal bases + emission histogram with the matrices of the current Z
            fill_ptc(w, -1, 0.0);
            uint64_t pos = w.st.pos;
            errs |= sample_pass(w, pos);
            pos += (uint64_t)w.tg_draws;
            PHASE(0);
            emission_sums(w);
            // missing nodes keep fixed emissions (bpp_c.hpp:451-474); the root has none
            for (int i = lane; i < N; i += 32) {
                if (w.missing[i]) { w.emis[i * 3 + 0] = 0; w.emis[i * 3 + 1] = d_log(dM.cons_to_mis); w.emis[i * 3 + 2] = 0; }
            }
            if (lane == 0) { w.emis[w.root * 3 + 0] = 0; w.emis[w.root * 3 + 1] = 0; w.emis[w.root * 3 + 2] = 0; }
            wsync();
            PHASE(1);
            errs |= update_z(w, pos);
            pos += (uint64_t)w.n_nodes;
            w.st.pos = pos;
            PHASE(2);
            // log-likelihood under the new Z when a branch changed (bpp_c.cpp:419-431)
            if (ancestors(w, 0, w.unv)) {
                fill_ptc(w, -1, 0.0);
                w.st.loglik = likelihood_pass(w, w.cur);
            }
            PHASE(3);
            // rates (bpp_c.cpp:434-452)
            double rn = mh_rate(w, true, w.trd[TR_N * T + m], m);
            if (lane == 0) w.trd[TR_N * T + m + 1] = rn;
            __syncwarp();
            PHASE(4);
            double rc = mh_rate(w, false, w.trd[TR_C * T + m], m);
            if (lane == 0) w.trd[TR_C * T + m + 1] = rc;
            PHASE(5);
            w.st.rate_n = rn;
            w.st.rate_c = rc;
            // transitions (sample_transition, bpp_c.cpp:522-613)
            double gr = 0, lr = 0, lr2 = 0;
            uint64_t p2 = w.st.pos;
            if (lane == 0) {
                double nZ[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                for (int k = 0; k + 1 < w.n_nodes; k++) {
                    int s = w.nodes[k];
                    nZ[w.Z[s]][w.Z[w.par[s]]] += 1;
                }
                StreamReader rd;
                rd.init(dM.seed, p2);
                gr = rd.beta(dM.ga + nZ[1][0] + nZ[2][0], dM.gb + nZ[0][0]);
                for (int k = 0; k + 1 < w.n_nodes; k++) {
                    int s = w.nodes[k];
                    if (w.fixZ[s] == 1) nZ[w.Z[s]][w.Z[w.par[s]]] -= 1;
                }
                lr = rd.beta(dM.la + nZ[2][1], dM.lb + nZ[1][1]);
                lr2 = (dM.l2a == 0) ? 0.0 : rd.beta(dM.l2a + nZ[1][2], dM.l2b + nZ[2][2]);
                p2 = rd.pos;
                w.trd[TR_G * T + m + 1] = gr;
                w.trd[TR_L * T + m + 1] = lr;
                w.trd[TR_L2 * T + m + 1] = lr2;
            }
            w.st.gr = bcast(gr);
            w.st.lr = bcast(lr);
            w.st.lr2 = bcast(lr2);
            w.st.pos = bcast(p2);
            w.st.m = m + 1;
            w.st.iters++;
            budget--;
            __syncwarp();
        }
        if (errs) w.st.status |= 1;
        write_slot_z(w);
        if (lane == 0) *sp = w.st;
        unsigned long long ei = w.e_int, el = w.e_leaf, nt = w.n_tg;
        for (int o = 16; o > 0; o >>= 1) {
            ei += __shfl_xor_sync(0xffffffffu, ei, o);
            el += __shfl_xor_sync(0xffffffffu, el, o);
            nt += __shfl_xor_sync(0xffffffffu, nt, o);
        }
        if (lane == 0 && P.counters) {
            for (int q = 0; q < 8; q++) atomicAdd(&P.counters->phase_cycles[q], w.ph[q]);
            atomicAdd(&P.counters->edge_internal, ei);
            atomicAdd(&P.counters->edge_leaf, el);
            atomicAdd(&P.counters->tg_draws, nt);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// host-callable pieces
// ---------------------------------------------------------------------------
// The model is copied on the stream the kernels run on, so that a launch
// that follows on that stream sees it.
cudaError_t set_model_batch(const DevModel& m, cudaStream_t st) {
    return cudaMemcpyToSymbolAsync(dM, &m, sizeof(DevModel), 0, cudaMemcpyHostToDevice, st);
}

size_t batch_warp_smem(int N, int NI, int S, int D, int prec, int C) {
    return prec == 0 ? WarpSmem<double>::make(N, NI, S, D, C).total : WarpSmem<float>::make(N, NI, S, D, C).total;
}
size_t batch_slot_bytes(int N, int T) { return SlotLayout::make(N, T).total; }
size_t batch_grp_bytes(int mcmc, int NI, int prec, int GGuP, int N) {
    return GrpLayout::make(mcmc, NI, prec == 0 ? 8 : 4, GGuP, N).total;
}
size_t batch_state_bytes() { return sizeof(SlotState); }

// Slot states for a fresh batch: slot i runs element elem[i].
__global__ void init_slots_kernel(SlotState* s, const int32_t* elem, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    SlotState z;
    memset(&z, 0, sizeof(z));
    z.elem = elem[i];
    z.phase = elem[i] < 0 ? PH_EMPTY : PH_INIT;
    s[i] = z;
}

cudaError_t launch_init_slots(void* slots, const int32_t* elem, int n, cudaStream_t st) {
    init_slots_kernel<<<(n + 127) / 128, 128, 0, st>>>((SlotState*)slots, elem, n);
    return cudaGetLastError();
}

template <typename Real, int C>
static cudaError_t launch_batch_t(const BatchParams& p, int grid, int warps, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(batch_kernel<Real, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    batch_kernel<Real, C><<<grid, warps * 32, smem, st>>>(p);
    return cudaGetLastError();
}

template <typename Real, int C>
static int occupancy_t(int warps, size_t smem) {
    if (cudaFuncSetAttribute(batch_kernel<Real, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_kernel<Real, C>, warps * 32, smem) != cudaSuccess)
        return 0;
    return nb;
}

// Resident CTAs per SM of the batched kernel for this shape (0 if it cannot run).
int batch_occupancy(int prec, int C, int warps, size_t smem) {
    if (prec == 0) {
        if (C == 1) return occupancy_t<double, 1>(warps, smem);
        if (C == 2) return occupancy_t<double, 2>(warps, smem);
    } else {
        if (C == 1) return occupancy_t<float, 1>(warps, smem);
        if (C == 2) return occupancy_t<float, 2>(warps, smem);
        if (C == 4) return occupancy_t<float, 4>(warps, smem);
    }
    return 0;
}

// Column counts per lane that are compiled: FP32 1, 2, 4; FP64 1, 2.
bool batch_supports(int prec, int C) { return prec == 0 ? (C == 1 || C == 2) : (C == 1 || C == 2 || C == 4); }

cudaError_t launch_batch(const void* params, int grid, int warps, size_t smem, int prec, int C, cudaStream_t st) {
    const BatchParams& p = *(const BatchParams*)params;
    if (prec == 0) {
        if (C == 1) return launch_batch_t<double, 1>(p, grid, warps, smem, st);
        if (C == 2) return launch_batch_t<double, 2>(p, grid, warps, smem, st);
    } else {
        if (C == 1) return launch_batch_t<float, 1>(p, grid, warps, smem, st);
        if (C == 2) return launch_batch_t<float, 2>(p, grid, warps, smem, st);
        if (C == 4) return launch_batch_t<float, 4>(p, grid, warps, smem, st);
    }
    return cudaErrorInvalidValue;
}

size_t batch_params_bytes() { return sizeof(BatchParams); }

}  // namespace pacc
