// pacc_chain.cu — PhyloAcc-ST's per-element MCMC as one CUDA thread block
// per element (sm_103a).
//
// One CTA runs an element through M0, M1 and M2 (src/PhyloAcc-ST/main.cpp:468-494):
// initMCMC -> Gibbs -> Eval2 -> Output_init, all on the device.  The
// element's alignment columns are spread over the CTA's threads; every
// chain-level step (latent-state filter, Metropolis-Hastings decisions,
// Beta draws) is done by a few threads between block barriers.
//
// Numerics.  The reference keeps every partial likelihood in log space and
// combines children with a 4x4 log-sum-exp (BPP::log_multi, bpp.hpp:427-445).
// Here partials are linear, L_s[j] = prod_children sum_i P(j->i) L_c[i], kept
// as mantissa * 2^scale with an integer exponent per (node, column): the
// power-of-two rescale is exact, so the values equal the log-space ones up to
// rounding (about 1e-16 relative per column in FP64).  Skipped children (gap
// or missing, bpp_c.cpp:653,660) multiply by nothing, like the reference's
// "add nothing".
//
// Partial re-pruning follows the reference's visited masks
// (getUpdateNode, bpp_c.cpp:620-642, 836-858): only ancestors of changed
// branches are recomputed.  MH proposals write the recomputed nodes to the
// other half of a per-node double buffer (the reference's lambda_tmp,
// bpp_c.cpp:981-989) and an accepted proposal flips the buffer index of
// those nodes instead of copying (bpp_c.cpp:1083-1092).
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "pacc_common.cuh"

namespace pacc {

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}


// Workspace carve-up (per CTA).
struct WsLayout {
    size_t lam, scale, tg, trz, trd, hash, rep, cfg, nxt, head, first, cstat, codes, prefix, total;
    __host__ __device__ static WsLayout make(int n_int, int GGp, int T, int mcmc, int N, int real_bytes) {
        WsLayout w;
        size_t o = 0;
        auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
        w.lam = o; o = al(o + (size_t)2 * n_int * 4 * GGp * real_bytes);
        w.scale = o; o = al(o + (size_t)2 * n_int * GGp * 4);
        w.tg = o; o = al(o + (size_t)n_int * GGp);
        w.trz = o; o = al(o + (size_t)T * N);
        w.trd = o; o = al(o + (size_t)7 * T * 8);
        w.hash = o; o = al(o + (size_t)(mcmc + 1) * 8);
        w.rep = o; o = al(o + (size_t)(mcmc + 1) * 4);
        w.cfg = o; o = al(o + (size_t)(mcmc + 1) * 4);
        w.nxt = o; o = al(o + (size_t)(mcmc + 1) * 4);
        w.head = o; o = al(o + (size_t)(mcmc + 2) * 4);
        w.first = o; o = al(o + (size_t)(mcmc + 2) * 4);
        w.cstat = o; o = al(o + (size_t)9 * (mcmc + 2) * 8);
        w.codes = o; o = al(o + (size_t)N * GGp);          // stream mode: the element's codes [S][GGp]
        w.prefix = o; o = al(o + (size_t)(GGp + 1) * 4);   // stream mode: its draw prefix
        w.total = o;
        return w;
    }
};

// trace_d rows
enum { TR_LL = 0, TR_FULL = 1, TR_N = 2, TR_C = 3, TR_G = 4, TR_L = 5, TR_L2 = 6 };

// Chain scalars shared by the block.
struct ChainScalars {
    uint64_t pos;          // next stream word
    double rate_n, rate_c; // current rates
    double prop_n, prop_c;
    double loglik;         // log_lik_old
    double maxll;
    double proposal;
    double mh_new;
    int acc_n, acc_c;
    int m, resZ, mi;
    int max_m;
    int skip;              // proposal rejected before the likelihood
    int accept;
    int any_unv;
    int status;
    int n_unc, n_conf, eff;
    double vb;
    int fallback;
    int n_list;            // entries of the current pass's node list
    // FP32-partial path: logs kept with the rates so the monitor and the MH
    // ratios need at most two new logarithms per step
    double lcur_n, lcur_c; // log rate_n, log rate_c
    double lpn;            // log prop_n
    double lgn;            // lgamma(rate_n / prop_n), valid when lgn_ok
    int lgn_ok;
};

// Reduction scratch: one slot per warp (<= 32), the broadcast slot RED_SUM
// and the median slot RED_MED.
static const int RED_SUM = 80, RED_MED = 81, RED_SLOTS = 88;

// Slots of the sampling pass's ring of column data copied ahead into
// shared memory (cp.async): the nodes up to RING-1 steps ahead are in
// flight while a node is drawn.
static const int RING = 3;

// One internal node of a pruning pass (the nodes flagged for the pass, in
// the element's stack order: every node after its children, the child whose
// subtree needs more pending partials first).  Child slot 0 is the child
// visited second, whose partial is on top of the stack when both children
// were computed in the same pass.
enum { K_SKIP = 0, K_LEAF = 1, K_MEM = 2, K_STACK = 3 };
struct __align__(16) PNode {
    int32_t dst;        // row of the result: (buffer * n_int + rank) * GGp
    int32_t src[2];     // leaf child: codes row (leaf * GGp); K_MEM child: its partial row; else -1
    int32_t act[2];     // internal child: its activity row (rank * GGp); leaf: -1
    int16_t mat[2];     // the child's transition matrix: class * N + child
    int8_t kind[2];     // K_SKIP (missing child), K_LEAF, K_MEM (internal, unchanged in this pass), K_STACK
    int8_t push;        // the parent is in the pass: the result goes on the stack
    int8_t is_root;
    int32_t pad;
};

// One internal node of the sampling pass (root first, then the internal
// nodes in reverse postorder, so a parent's base is drawn before its
// children's).
struct __align__(16) SNode {
    int32_t part;       // partial row of the node in its current buffer: (cur * n_int + rank) * GGp
    int32_t act;        // activity row (rank * GGp); -1: a missing node (never drawn)
    int16_t mat;        // matrix of the node's own branch: class(Z) * N + node
    int16_t rank;       // base slot of the node
    int16_t prank;      // base slot of the parent (-1 for the root)
    int16_t node;       // emission row of the node's branch (-1: the root or a missing node)
    int16_t leaf[2];    // leaf children whose branches emit under this node (-1: none or missing)
    int32_t pad[2];
};

// Shared-memory layout (dynamic, sized by N, the block size and the
// prune's stack depth D).
template <typename Real>
struct SmemLayout {
    size_t ptd, ptr_, ltm, emis, beta, cnt, red, i16, i8, dist, scr, ring, stks, desc, total;
    __host__ __device__ static SmemLayout make(int N, int BT, int D) {
        SmemLayout s;
        size_t o = 0;
        auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
        const int n_int = (N + 1) / 2 - 1 > 0 ? (N + 1) / 2 - 1 : 1;   // internal nodes of a binary tree
        // column scratch of one pass, per thread: the internal bases of its
        // column and the ring of prefetched partials (sampling pass), or the
        // stack of pending partials and their scales (prune)
        const size_t sb = al((size_t)n_int * BT) + (size_t)RING * BT * (4 * sizeof(Real) + 12);
        const size_t sk = al((size_t)D * BT * 4 * sizeof(Real)) + (size_t)D * BT * 4;
        s.scr = o; o = al(o + (sb > sk ? sb : sk));
        s.ring = s.scr + al((size_t)n_int * BT);
        s.stks = s.scr + al((size_t)D * BT * 4 * sizeof(Real));
        s.desc = o; o = al(o + (size_t)n_int * 32);                              // PNode / SNode list
        s.dist = o; o = al(o + (size_t)N * 8);                                   // branch lengths
        // P^T per class [4][N][16]: FP64 for FP64 partials; FP32 partials keep
        // only the FP32 copy (the FP64 product is formed in registers)
        s.ptd = o; o = al(o + (sizeof(Real) == 8 ? (size_t)4 * N * 16 * 8 : 0));
        s.ptr_ = o; o = al(o + (sizeof(Real) == 8 ? 0 : (size_t)4 * N * 16 * sizeof(Real)));
        s.ltm = o; o = al(o + (sizeof(Real) == 8 ? (size_t)N * 9 * 8 : 0));  // log_TM_Int [N][3][3] (FP64 path)
        s.emis = o; o = al(o + (size_t)N * 3 * 8);
        s.beta = o; o = al(o + (size_t)N * 3 * 8);
        s.cnt = o; o = al(o + (size_t)N * NSYM * 2 * 4);                    // emission histogram (16-bit bins)
        s.red = o; o = al(o + (size_t)RED_SLOTS * 8);                        // reduction scratch
        s.i16 = o; o = al(o + (size_t)TopoLayout::make(N).total * 2);
        s.i8 = o; o = al(o + (size_t)N * 8);                               // Z fixZ changed unv unvN unvC cur maxz
        s.total = o;
        return s;
    }
};

enum { P_NULL = 0, P_CONS = 1, P_NEUT = 2, P_PROP = 3 };


// ---------------------------------------------------------------------------
// Small helpers
// ---------------------------------------------------------------------------
// Exact sum of per-column log-likelihoods.  Each column's FP64 value v is
// held exactly in 64.64 fixed point (floor(v) and the 64-bit fraction
// (v - floor(v)) * 2^64; exact for |v| >= 2^-12, below that the bits under
// 2^-64 are dropped) and added in 128-bit integers, which is associative: the
// total does not depend on how columns are spread over threads, and it is
// the exact sum of the column values rounded once (more than the Kahan
// compensation of an FP64 running sum gives).  A column of -inf or NaN makes
// the total -inf or NaN, as log-sum-exp accumulation does.
struct ColSum {
    __int128 acc;
    int bad;      // bit 0: a -inf column; bit 1: a NaN or +inf column
    __device__ __forceinline__ void init() { acc = 0; bad = 0; }
    __device__ __forceinline__ void add(double v) {
        if (!(v > -CUDART_INF && v < CUDART_INF)) {
            bad |= (v == -CUDART_INF) ? 1 : 2;
            return;
        }
        const double h = floor(v);
        const long long hi = (long long)h;
        const unsigned long long lo = (unsigned long long)((v - h) * 18446744073709551616.0);
        acc += ((__int128)hi << 64) + (__int128)lo;
    }
};

// Block-wide total of the threads' ColSums (every thread gets the result).
__device__ __forceinline__ double block_colsum(ColSum s, double* red) {
    unsigned long long lo = (unsigned long long)s.acc;
    long long hi = (long long)(s.acc >> 64);
    int bad = s.bad;
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long lo2 = __shfl_down_sync(0xffffffffu, lo, o);
        const long long hi2 = __shfl_down_sync(0xffffffffu, hi, o);
        bad |= __shfl_down_sync(0xffffffffu, bad, o);
        const __int128 t = (((__int128)hi << 64) | lo) + (((__int128)hi2 << 64) | lo2);
        lo = (unsigned long long)t;
        hi = (long long)(t >> 64);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    unsigned long long* r64 = (unsigned long long*)red;   // [warp][lo, hi], then the flags
    int* rbad = (int*)(r64 + 2 * 32);
    __syncthreads();
    if (l == 0) {
        r64[2 * w] = lo;
        r64[2 * w + 1] = (unsigned long long)hi;
        rbad[w] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __int128 t = 0;
        int b = 0;
        const int nw = blockDim.x >> 5;
        for (int i = 0; i < nw; i++) {
            t += ((__int128)(long long)r64[2 * i + 1] << 64) | r64[2 * i];
            b |= rbad[i];
        }
        double v = (double)(long long)(t >> 64) + (double)(unsigned long long)t * 0x1p-64;
        if (b & 2) v = CUDART_NAN;
        else if (b & 1) v = -CUDART_INF;
        red[RED_SUM] = v;
    }
    __syncthreads();
    const double v = red[RED_SUM];
    __syncthreads();
    return v;
}

__device__ __forceinline__ int block_or(int v, int* tmp) {
    __syncthreads();
    if (threadIdx.x == 0) *tmp = 0;
    __syncthreads();
    if (v) atomicOr(tmp, 1);
    __syncthreads();
    int r = *tmp;
    __syncthreads();
    return r;
}

// Exact rescale by a power of two when the largest entry is small.
template <typename Real> struct Rescale;
template <> struct Rescale<double> {
    static __device__ __forceinline__ void apply(double* a, int& sc) {
        double mx = fmax(fmax(a[0], a[1]), fmax(a[2], a[3]));
        if (mx < 0x1p-256 && mx > 0) {
            do {
#pragma unroll
                for (int j = 0; j < 4; j++) a[j] *= 0x1p256;
                sc -= 256;
                mx *= 0x1p256;
            } while (mx < 0x1p-256);
        }
    }
};
template <> struct Rescale<float> {
    static __device__ __forceinline__ void apply(float* a, int& sc) {
        float mx = fmaxf(fmaxf(a[0], a[1]), fmaxf(a[2], a[3]));
        if (mx < 0x1p-60f && mx > 0) {
            int e;
            frexpf(mx, &e);
            // bring the max into [0.5, 1): multiply by 2^(-e) in two exact steps
            int k = -e;
            float f1 = ldexpf(1.0f, k / 2), f2 = ldexpf(1.0f, k - k / 2);
#pragma unroll
            for (int j = 0; j < 4; j++) a[j] = (a[j] * f1) * f2;
            sc -= k;
        }
    }
};

// ---------------------------------------------------------------------------
// The element context held by one CTA
// ---------------------------------------------------------------------------
template <typename Real>
struct Ctx {
    // element
    int S, N, GG, GGp, root, n_nodes, n_int, n_hlev, n_dlev, tg_draws;
    const uint8_t* codes;     // [S][GGp]
    const int32_t* prefix;    // [GG+1]
    // topology in shared
    int16_t *nodes, *internal, *c2a, *c2b, *par, *irank, *pos, *missing, *upc, *upcc, *hlev_start, *hlev_nodes,
        *dlev_start, *dlev_nodes;
    int16_t *sord, *sflag;
    // shared state
    double* ptd;              // [4][N][16] (FP64 partials only; null for FP32)
    Real* ptr;                // [4][N][16]
    double* ltm;              // [N][9] log_TM_Int (zc*3+zp)
    double* emis;             // [N][3]
    double* beta;             // [N][3]
    unsigned* cnt;            // [N][NSYM*2]: (child symbol, parent base) counts, two 16-bit bins a word
    double* red;
    int8_t *Z, *fixZ, *changed, *unv, *unvN, *unvC, *cur, *maxz;
    ChainScalars* cs;
    int8_t* bases;            // sampling pass: [n_int][BT] internal bases of each thread's column
    Real* ring;               // sampling pass: [RING][BT][4] partials copied ahead, then [RING][3][BT]
                              // words holding the activity byte and two leaf codes
    Real* stk;                // prune: [D][BT][4] pending partials
    int32_t* stks;            // prune: [D][BT] their scales
    PNode* pn;                // the pass's node list
    SNode* sn;
    int D;                    // stack rows
    // workspace
    Real* lam;                // [2][n_int][GGp][4] partials, one 4-vector per (node, column)
    int32_t* scl;             // [2][n_int][GGp] their power-of-two exponents
    int8_t* act;              // [n_int][GGp] static: < 4 where an internal node is sampled and pruned
                              // (the initial Tg; 4 where both children are gaps or missing)
    int8_t* trz;              // [T][N]
    double* trd;              // [7][T]
    uint64_t* hash;
    int32_t *rep, *cfg, *nxt, *head, *first;
    double* cstat;
    int T, burn, mcmc;
    DevCounters local;
};

// One partial 4-vector: 16-byte (FP32) or two 16-byte (FP64) accesses.
__device__ __forceinline__ void ld4(const float* p, float (&x)[4]) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&x)[4]) {
    const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
    x[0] = a.x; x[1] = a.y; x[2] = b.x; x[3] = b.y;
}
__device__ __forceinline__ void st4(float* p, const float (&x)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(x[0], x[1], x[2], x[3]);
}
__device__ __forceinline__ void st4(double* p, const double (&x)[4]) {
    reinterpret_cast<double2*>(p)[0] = make_double2(x[0], x[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(x[2], x[3]);
}

// Class of the matrix used for child c: Z 2 -> neut, 0 -> null, else cons
// (bpp_c.cpp:661-663); in an MH proposal the proposed class uses P_PROP (bpp_c.cpp:885-906).
__device__ __forceinline__ int mat_class(int z, int prop_class) {
    int k = (z == 2) ? P_NEUT : (z == 0 ? P_NULL : P_CONS);
    return (prop_class >= 0 && k == prop_class) ? P_PROP : k;
}

// One row of a 4x4 matrix (16-byte aligned rows: matrices are 16 entries
// apart from an aligned base).
__device__ __forceinline__ void ld_row(const float* p, float (&r)[4]) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
}
__device__ __forceinline__ void ld_row(const double* p, double (&r)[4]) {
    const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
    r[0] = a.x; r[1] = a.y; r[2] = b.x; r[3] = b.y;
}

// The pass's node list for a prune over the nodes flagged in `unv`: the
// flagged, non-missing internal nodes in stack order, with their children
// resolved (data source, matrix, stack use).  Built by warp 0 with a ballot
// compaction, so the column loop reads one 32-byte entry per node.
// mh = false: results overwrite the current buffer of each node (Update_Tg
// with visited masks, bpp_c.cpp:647-671).  mh = true: results go to the other
// buffer (log_f_Xz into lambda_tmp, bpp_c.cpp:860-928), and the children in
// class prop_class take the proposal's matrices (bpp_c.cpp:885-906).
// The flagged sets of every pass are closed upwards (ancestors of changed
// branches, getUpdateNode), so every pushed partial is popped by its parent.
template <typename Real>
__device__ int build_prune_list(Ctx<Real>& c, const int8_t* unv, bool mh, int prop_class) {
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        int base = 0;
        for (int k0 = 0; k0 < c.n_int; k0 += 32) {
            const int k = k0 + lane;
            int s = -1;
            bool f = false;
            if (k < c.n_int) {
                s = c.sord[k];
                f = unv[s] && !c.missing[s];
            }
            const unsigned b = __ballot_sync(0xffffffffu, f);
            if (f) {
                PNode d;
                const int ir = c.irank[s];
                const int dbuf = mh ? 1 - c.cur[s] : c.cur[s];
                d.dst = (dbuf * c.n_int + ir) * c.GGp;
                d.is_root = (s == c.root);
                const int ps = c.par[s];
                d.push = (s != c.root && ps >= 0 && ps < c.N && unv[ps] && !c.missing[ps]) ? 1 : 0;
                // slot 0: the child visited second (top of the stack)
                const int a = c.c2a[s], bb = c.c2b[s];
                const int chs[2] = {c.sflag[s] ? a : bb, c.sflag[s] ? bb : a};
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const int ch = chs[q];
                    d.mat[q] = (int16_t)(mat_class(c.Z[ch], prop_class) * c.N + ch);
                    if (c.missing[ch]) {
                        d.kind[q] = K_SKIP; d.src[q] = -1; d.act[q] = -1;
                    } else if (ch < c.S) {
                        d.kind[q] = K_LEAF; d.src[q] = ch * c.GGp; d.act[q] = -1;
                    } else {
                        const int cir = c.irank[ch];
                        d.act[q] = cir * c.GGp;
                        if (unv[ch]) { d.kind[q] = K_STACK; d.src[q] = -1; }
                        else { d.kind[q] = K_MEM; d.src[q] = (c.cur[ch] * c.n_int + cir) * c.GGp; }
                    }
                }
                d.pad = 0;
                c.pn[base + __popc(b & ((1u << lane) - 1u))] = d;
            }
            base += __popc(b);
        }
        if (lane == 0) c.cs->n_list = base;
    }
    __syncthreads();
    return c.cs->n_list;
}

// What a column needs of one child before the arithmetic: issued for the
// next node while the current one is computed (none of it depends on the
// pass's own results).
template <typename Real>
struct ChildCol {
    Real x[4];
    int code;     // leaf: column code; internal: activity (< 4 = active)
    int sc;
};

template <typename Real>
__device__ __forceinline__ void load_child(const Ctx<Real>& c, const PNode& d, int q, int g, ChildCol<Real>& o) {
    o.sc = 0;
    o.code = 4;
    const int kd = d.kind[q];
    if (kd == K_LEAF) {
        o.code = c.codes[d.src[q] + g];
    } else if (kd >= K_MEM) {
        o.code = c.act[d.act[q] + g];
        if (kd == K_MEM) {
            ld4(c.lam + ((size_t)d.src[q] + g) * 4, o.x);
            o.sc = c.scl[d.src[q] + g];
        }
    }
}

// Felsenstein pruning over the flagged nodes (see build_prune_list), all
// columns; returns the summed per-column log-likelihood at the root (valid
// when the root is flagged).  A thread walks its column through the list:
// partials computed in this pass are passed to the parent through a
// shared-memory stack of depth D (the element's stack order bounds it), and
// only unchanged children are read from the partial buffers.
template <typename Real>
__device__ double prune(Ctx<Real>& c, const int8_t* unv, bool mh, int prop_class) {
    const int n = build_prune_list(c, unv, mh, prop_class);
    const int BT = blockDim.x, tid = threadIdx.x;
    ColSum ll;
    ll.init();
    unsigned long long e_int = 0, e_leaf = 0;
    int overflow = 0;
    for (int g = tid; g < c.GG; g += BT) {
        int sp = 0;
        PNode dn = c.pn[0];
        ChildCol<Real> n0, n1;
        if (n > 0) { load_child(c, dn, 0, g, n0); load_child(c, dn, 1, g, n1); }
        for (int k = 0; k < n; k++) {
            const PNode d = dn;
            ChildCol<Real> ch[2] = {n0, n1};
            if (k + 1 < n) {
                dn = c.pn[k + 1];
                load_child(c, dn, 0, g, n0);
                load_child(c, dn, 1, g, n1);
            }
            Real a[4] = {1, 1, 1, 1};
            int sc = 0;
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int kd = d.kind[q];
                if (kd == K_SKIP) continue;
                const Real* PM = c.ptr + (size_t)d.mat[q] * 16;
                if (kd == K_LEAF) {
                    const int code = ch[q].code;
                    if (code == CODE_GAP || code == CODE_OTHER) continue;
                    if (code < 4) {
                        Real r[4];
                        ld_row(PM + code * 4, r);
#pragma unroll
                        for (int j = 0; j < 4; j++) a[j] *= r[j];
                    } else {
                        const int msk = ambig_mask(code - CODE_R);
                        Real v[4] = {0, 0, 0, 0};
#pragma unroll
                        for (int i = 0; i < 4; i++)
                            if (msk & (1 << i)) {
#pragma unroll
                                for (int j = 0; j < 4; j++) v[j] += PM[i * 4 + j];
                            }
#pragma unroll
                        for (int j = 0; j < 4; j++) a[j] *= v[j];
                    }
                    e_leaf++;
                } else {
                    if (kd == K_STACK) {
                        // the child's partial of this pass (on top of the stack)
                        if (sp > 0) {
                            sp--;
                            ld4(c.stk + ((size_t)sp * BT + tid) * 4, ch[q].x);
                            ch[q].sc = c.stks[sp * BT + tid];
                        } else {
                            overflow = 1;
                        }
                    }
                    if (ch[q].code >= KB) continue;
                    Real r0[4], r1[4], r2[4], r3[4];
                    ld_row(PM, r0); ld_row(PM + 4, r1); ld_row(PM + 8, r2); ld_row(PM + 12, r3);
                    const Real* x = ch[q].x;
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        Real v = r0[j] * x[0];
                        v += r1[j] * x[1];
                        v += r2[j] * x[2];
                        v += r3[j] * x[3];
                        a[j] *= v;
                    }
                    sc += ch[q].sc;
                    e_int++;
                }
            }
            Rescale<Real>::apply(a, sc);
            if (d.is_root) {
#pragma unroll
                for (int j = 0; j < 4; j++) a[j] *= (Real)dM.pi[j];
                const double t = (double)a[0] + (double)a[1] + (double)a[2] + (double)a[3];
                if (sizeof(Real) == 8) {
                    ll.add(d_log(t) + (double)sc * 0.6931471805599453);
                } else {
                    // FP32 partials: the column's log from its FP64 root sum
                    // t = m 2^e as (e + scale) ln 2 + log m, log m in FP32 (the
                    // partials carry FP32 rounding already)
                    int e1;
                    const double mt = frexp(t, &e1);
                    ll.add(t > 0 ? (double)(e1 + sc) * 0.6931471805599453 + (double)logf((float)mt)
                                 : (t == 0 ? -CUDART_INF : CUDART_NAN));
                }
            }
            st4(c.lam + ((size_t)d.dst + g) * 4, a);
            c.scl[d.dst + g] = sc;
            if (d.push) {
                if (sp < c.D) {
                    st4(c.stk + ((size_t)sp * BT + tid) * 4, a);
                    c.stks[sp * BT + tid] = sc;
                } else {
                    overflow = 1;
                }
                sp++;
            }
        }
    }
    if (overflow) atomicOr(&c.cs->status, 1);
    c.local.edge_internal += e_int;
    c.local.edge_leaf += e_leaf;
    double r = block_colsum(ll, c.red);
    if (threadIdx.x == 0) c.local.col_ll += c.GG;
    return r;
}

// P^T(d r) of the FP32-partial path: the exponentials exp(lambda_i d r) in
// FP64, then the 4x4 product in FP32 as I + sum_i A_i (exp(lambda_i d r) - 1)
// with A_i = eigeninv[:, i] eigenvec[i, :].  Its terms are of the size of the
// result, so the small entries of short branches do not come from
// cancelling O(1) terms (as they would in eigeninv diag(e) eigenvec).
static __device__ __noinline__ void build_pt32(double d, double r, bool scaled, float* out) {
    float em1[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        double x = __dmul_rn(dM.lam[i], d);
        if (scaled) x = __dmul_rn(x, r);
        em1[i] = (float)(d_exp(x) - 1.0);
    }
#pragma unroll
    for (int ab = 0; ab < 16; ab++) {
        const float* A = dM.a32 + ab * 4;
        float s = A[0] * em1[0];
        s = fmaf(A[1], em1[1], s);
        s = fmaf(A[2], em1[2], s);
        s = fmaf(A[3], em1[3], s);
        out[ab] = s + (((ab >> 2) == (ab & 3)) ? 1.0f : 0.0f);
    }
}

// P^T of class k for node s at rate r.  Branches shorter than 1e-10 keep the
// identity (bpp_c.cpp:191-226, 1123) unless force_eigen: the proposal
// matrices of log_f_Xz (bpp_c.cpp:887-902) and the Eval2 fallback
// (bpp_c2.cpp:220-237) apply the eigen formula whatever the branch length.
template <typename Real>
__device__ __forceinline__ void build_one(Ctx<Real>& c, const double* dist2, int k, int s, double r, bool scaled,
                                          bool force_eigen) {
    const bool eig = force_eigen || dist2[s] > 1e-10;
    if (sizeof(Real) == 8) {
        double* out = c.ptd + ((size_t)k * c.N + s) * 16;
        if (eig) build_pt(dist2[s], r, scaled, out);
        else identity_pt(out);
    } else {
        float* out = (float*)c.ptr + ((size_t)k * c.N + s) * 16;
        if (eig) build_pt32(dist2[s], r, scaled, out);
        else {
#pragma unroll
            for (int q = 0; q < 16; q++) out[q] = ((q >> 2) == (q & 3)) ? 1.0f : 0.0f;
        }
    }
    c.local.pmat++;
}

// The P^T table of class k for all nodes of the pruned tree (except the root).
template <typename Real>
__device__ void build_class(Ctx<Real>& c, const double* dist2, int k, double r, bool scaled, bool force_eigen) {
    for (int i = threadIdx.x; i < c.n_nodes - 1; i += blockDim.x) build_one(c, dist2, k, c.nodes[i], r, scaled, force_eigen);
}

// The proposal's matrices (log_f_Xz, bpp_c.cpp:885-906) for the branches a
// proposal of class cls changes: those whose Z puts them in the class.  The
// prune reads the proposal's matrices for exactly these children.
template <typename Real>
__device__ void build_prop(Ctx<Real>& c, const double* dist2, int cls, double r) {
    for (int i = threadIdx.x; i < c.n_nodes - 1; i += blockDim.x) {
        const int s = c.nodes[i];
        if (mat_class(c.Z[s], -1) == cls) build_one(c, dist2, P_PROP, s, r, true, true);
    }
}

// An accepted proposal becomes the class's cache (bpp_c.cpp:1115-1131): the
// branches that took the proposal's matrices keep them, the others get the
// same matrices at the new rate; branches shorter than 1e-10 are not rebuilt
// (bpp_c.cpp:1123).
template <typename Real>
__device__ void accept_class(Ctx<Real>& c, const double* dist2, int cls, double r) {
    for (int i = threadIdx.x; i < c.n_nodes - 1; i += blockDim.x) {
        const int s = c.nodes[i];
        if (dist2[s] < 1e-10) continue;
        if (mat_class(c.Z[s], -1) == cls) {
            const Real* a = c.ptr + ((size_t)P_PROP * c.N + s) * 16;
            Real* b = c.ptr + ((size_t)cls * c.N + s) * 16;
#pragma unroll
            for (int q = 0; q < 16; q++) b[q] = a[q];
        } else {
            build_one(c, dist2, cls, s, r, true, true);
        }
    }
}

// log_TM_Int from the current g, l, l2 (bpp_c.cpp:301-332, 573-599).
// Only the log-space Z filter of the FP64 path reads it; the FP32 path's
// linear filter forms its transition matrix from g, l and l2 directly.
template <typename Real>
__device__ void build_ltm(Ctx<Real>& c, double gr, double lr, double lr2, bool init) {
    if (sizeof(Real) != 8) return;
    const double NI = -CUDART_INF;
    // the six logs depend on g, l and l2 only: one evaluation each
    const double lg0 = d_log(1 - gr), lg1 = d_log(gr);
    const double y = 1 - lr;
    const double ll1 = d_log(y), ll2 = d_log(1 - y);
    const double lm1 = d_log(lr2), lm2 = d_log(1 - lr2);
    for (int i = threadIdx.x; i < c.n_nodes; i += blockDim.x) {
        int s = c.nodes[i];
        double* t = c.ltm + (size_t)s * 9;   // t[zc*3 + zp]
        if (c.fixZ[s] == 1) {
            if (init) {
                t[0 * 3 + 1] = NI;
                // parent state 2 never occurs above a fixed node; the
                // reference's matrix keeps its initial zeros there
                t[0 * 3 + 2] = 0;
                t[1 * 3 + 2] = 0;
                t[2 * 3 + 2] = 0;
            }
            t[1 * 3 + 1] = 0;
            t[2 * 3 + 1] = NI;
            t[0 * 3 + 0] = lg0;
            t[1 * 3 + 0] = lg1;
            t[2 * 3 + 0] = NI;
        } else {
            t[0 * 3 + 0] = lg0;
            t[1 * 3 + 0] = lg1;
            t[2 * 3 + 0] = NI;
            if (init) t[0 * 3 + 1] = NI;
            t[1 * 3 + 1] = ll1;
            t[2 * 3 + 1] = ll2;
            if (init) t[0 * 3 + 2] = NI;
            t[1 * 3 + 2] = lm1;
            t[2 * 3 + 2] = lm2;
        }
    }
}

// The sampling pass's node list: the root, then the internal nodes in
// reverse postorder (internal[n_int-2] .. internal[0]), each with its
// partial row in the current buffer, the matrix of its branch and the
// leaf children whose branch emissions are counted under it.
template <typename Real>
__device__ void build_sample_list(Ctx<Real>& c) {
    __syncthreads();
    for (int i = threadIdx.x; i < c.n_int; i += blockDim.x) {
        const int s = c.internal[c.n_int - 1 - i];
        const int ir = c.irank[s];
        SNode d;
        d.part = (c.cur[s] * c.n_int + ir) * c.GGp;
        const bool miss = c.missing[s] != 0;
        d.act = miss ? -1 : ir * c.GGp;
        d.mat = (int16_t)(mat_class(c.Z[s], -1) * c.N + s);
        d.rank = (int16_t)ir;
        d.prank = (int16_t)(s == c.root ? -1 : c.irank[c.par[s]]);
        d.node = (int16_t)((s == c.root || miss) ? -1 : s);
        const int a = c.c2a[s], b = c.c2b[s];
        d.leaf[0] = (int16_t)((a >= 0 && a < c.S && !c.missing[a]) ? a : -1);
        d.leaf[1] = (int16_t)((b >= 0 && b < c.S && !c.missing[b]) ? b : -1);
        d.pad[0] = d.pad[1] = 0;
        c.sn[i] = d;
    }
    for (int i = threadIdx.x; i < c.N * NSYM * 2; i += blockDim.x) c.cnt[i] = 0;
    __syncthreads();
}

// One histogram count for the branch above `row`: one shared atomic per
// lane (the hardware merges a warp's atomics on one address; merging them
// first with match_any or ballots measured slower).  Bins are 16 bits, two to
// a word (a branch counts at most one pair per column, and elements have
// fewer than 65,536 columns).
__device__ __forceinline__ void emit_key(unsigned* cnt, int row, int key) {
    if (key >= 0) atomicAdd(&cnt[row * (NSYM * 2) + (key >> 1)], 1u << (16 * (key & 1)));
}
__device__ __forceinline__ int bin_count(const unsigned* cnt, int row, int key) {
    return (int)((cnt[row * (NSYM * 2) + (key >> 1)] >> (16 * (key & 1))) & 0xffffu);
}

// Asynchronous 16-byte global -> shared copies (cp.async, L2 only).
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async4(void* sdst, const void* gsrc) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gsrc) : "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }
// One partial 4-vector (16 or 32 bytes).
__device__ __forceinline__ void cp_part(float* sdst, const float* gsrc) { cp_async16(sdst, gsrc); }
__device__ __forceinline__ void cp_part(double* sdst, const double* gsrc) {
    cp_async16(sdst, gsrc);
    cp_async16(sdst + 2, gsrc + 2);
}

// Emission symbol of a leaf code: bases 0..3, ambiguity codes 4..9, else -1.
__device__ __forceinline__ int leaf_sym(int code) { return code < 4 ? code : (code >= CODE_R ? code - 2 : -1); }

// Internal-base sampling, top-down per column (Update_Tg with tosample,
// bpp_c.cpp:672-733), fused with the histogram of (child symbol, parent
// base) pairs of every branch that the emissions are summed from
// (getEmission, bpp_c2.cpp:355-390).  Column g takes its stream words at
// pos + prefix[g].  A thread keeps the bases of its column in shared memory
// (the parent's base is read there, not from device memory), loads the next
// node's partial while the current node is drawn, and the histogram counts
// are integers, so the order of the adds does not matter.  Each internal
// node's base is drawn afresh from the current partials, so bases need not
// outlive the pass: which nodes are drawn (and pruned) at a column is the
// static activity row.
template <typename Real>
__device__ int sample_emit(Ctx<Real>& c, uint64_t pos) {
    build_sample_list(c);
    int err = 0;
    const int BT = blockDim.x, tid = threadIdx.x;
    unsigned long long draws = 0;
    int8_t* bs = c.bases;
    const int n = c.n_int;
    // ring slot q of this thread: the partial, and the 4-byte words holding
    // the activity byte and the two leaf codes of the node RING-1 steps ahead
    Real* rp = c.ring;
    unsigned* rw = (unsigned*)(c.ring + (size_t)RING * BT * 4);
    for (int gb = 0; gb < c.GG; gb += BT) {
        const int g = gb + tid;
        const bool on = g < c.GG;
        const int gw = g & ~3, sh = 8 * (g & 3);
        // copies of node i's column data into ring slot i % RING
        auto issue = [&](int i) {
            if (on && i < n) {
                const SNode e = c.sn[i];
                const int q = i % RING;
                cp_part(rp + ((size_t)q * BT + tid) * 4, c.lam + ((size_t)e.part + g) * 4);
                if (e.act >= 0) cp_async4(rw + (q * 3 + 0) * BT + tid, c.act + e.act + gw);
                if (e.leaf[0] >= 0) cp_async4(rw + (q * 3 + 1) * BT + tid, c.codes + (size_t)e.leaf[0] * c.GGp + gw);
                if (e.leaf[1] >= 0) cp_async4(rw + (q * 3 + 2) * BT + tid, c.codes + (size_t)e.leaf[1] * c.GGp + gw);
            }
            cp_async_commit();
        };
        for (int i = 0; i < RING - 1; i++) issue(i);
        uint64_t w = on ? pos + (uint64_t)c.prefix[g] : 0;
        uint64_t blk = ~0ull;
        // the block's four words in scalars (an array indexed by w & 3 would
        // live in local memory)
        uint32_t w0 = 0, w1 = 0, w2 = 0, w3 = 0;
        auto next_word = [&]() {
            const uint64_t b = w >> 2;
            if (b != blk) {
                uint32_t o[4];
                philox4x32_10((uint32_t)b, (uint32_t)(b >> 32), 0u, 0u, dM.seed, 0u, o);
                w0 = o[0]; w1 = o[1]; w2 = o[2]; w3 = o[3];
                blk = b;
            }
            const int i = (int)(w++ & 3);
            return i == 0 ? w0 : (i == 1 ? w1 : (i == 2 ? w2 : w3));
        };
        // the draw: FP64 for FP64 partials (as the oracle), FP32 for FP32 partials
        auto draw4 = [&](const Real* q) -> int {
            const uint32_t wd = next_word();
            if (sizeof(Real) == 8) return categorical(4, q, word_to_uniform(wd));
            const float u = ((float)(wd >> 8) + 0.5f) * 5.9604644775390625e-08f;
            const float tot = ((float)q[0] + (float)q[1]) + ((float)q[2] + (float)q[3]);
            const float t = u * tot;
            // the first k with t < cum_k, from three compares (cum is non-decreasing)
            const float c0 = (float)q[0], c1 = c0 + (float)q[1], c2 = c1 + (float)q[2], c3 = c2 + (float)q[3];
            if (t < c3) return (t >= c0) + (t >= c1) + (t >= c2);
            for (int k = 3; k >= 0; k--)
                if (q[k] > 0) return k;
            return 4;
        };
        // node i = 0 is the root (always drawn), then the internal nodes top-down
        for (int i = 0; i < n; i++) {
            issue(i + RING - 1);
            cp_async_wait<RING - 1>();   // node i's copies have landed
            const SNode d = c.sn[i];
            const int q = i % RING;
            Real x[4];
            ld4(rp + ((size_t)q * BT + tid) * 4, x);
            const int a = (d.act >= 0 && i > 0) ? (int)((rw[(q * 3 + 0) * BT + tid] >> sh) & 0xff) : 0;
            const int lc0 = d.leaf[0] >= 0 ? (int)((rw[(q * 3 + 1) * BT + tid] >> sh) & 0xff) : 4;
            const int lc1 = d.leaf[1] >= 0 ? (int)((rw[(q * 3 + 2) * BT + tid] >> sh) & 0xff) : 4;
            int tp = 0, nb = 4;
            if (i == 0) {
                if (on) {
                    nb = draw4(x);
                    draws++;
                    if (nb > 3) { err = 1; nb = 0; }
                }
            } else {
                const bool drawn = on && d.act >= 0 && (int8_t)a < KB;
                tp = bs[d.prank * BT + tid];
                if (drawn) {
                    const Real* P = c.ptr + (size_t)d.mat * 16;
                    Real qv[4];
#pragma unroll
                    for (int k = 0; k < 4; k++) qv[k] = P[k * 4 + tp] * x[k];
                    nb = draw4(qv);
                    draws++;
                    if (nb > 3) { err = 1; nb = 0; }
                }
            }
            bs[d.rank * BT + tid] = (int8_t)nb;
            if (d.node >= 0) emit_key(c.cnt, d.node, (on && nb < KB && tp < KB) ? nb * 4 + tp : -1);
            if (d.leaf[0] >= 0) {
                const int sy = leaf_sym(lc0);
                emit_key(c.cnt, d.leaf[0], (on && sy >= 0 && nb < KB) ? sy * 4 + nb : -1);
            }
            if (d.leaf[1] >= 0) {
                const int sy = leaf_sym(lc1);
                emit_key(c.cnt, d.leaf[1], (on && sy >= 0 && nb < KB) ? sy * 4 + nb : -1);
            }
        }
        cp_async_wait<0>();
    }
    c.local.tg_draws += draws;
    __syncthreads();
    return err;
}

// Emission sums per branch and class (getEmission, bpp_c2.cpp:355-390) from
// the histogram of the sampling pass: e_s[z] = sum of counts * log P^T_z.
template <typename Real>
__device__ void emission(Ctx<Real>& c) {
    const int NB = NSYM * 4;
    for (int i = threadIdx.x; i < (c.n_nodes - 1) * 3; i += blockDim.x) {
        int s = c.nodes[i / 3];
        int z = i % 3;
        if (c.missing[s]) continue;
        const int cls = z == 0 ? P_NULL : (z == 1 ? P_CONS : P_NEUT);
        const Real* P = c.ptr + ((size_t)cls * c.N + s) * 16;
        double e = 0;
        for (int b = 0; b < NB; b++) {
            int n = bin_count(c.cnt, s, b);
            if (!n) continue;
            int sym = b >> 2, tp = b & 3;
            double t;
            if (sym < 4) t = P[sym * 4 + tp];
            else {
                int msk = ambig_mask(sym - 4);
                t = 0;
                for (int q = 0; q < 4; q++)
                    if (msk & (1 << q)) t += P[q * 4 + tp];
            }
            // with FP32 partials the log of the entry is taken in FP32 (the
            // emissions feed the Z filter, whose normalisation stays FP64)
            const double v = (sizeof(Real) == 8) ? d_log(t) : (double)f_log((float)t);
            e += (double)n * v;
        }
        c.emis[s * 3 + z] = e;
    }
    __syncthreads();
}

// log_multi2 column zp for child s (bpp.hpp:447-460)
__device__ __forceinline__ double msg(const double* ltm, const double* beta, int s, int zp) {
    double t0 = ltm[s * 9 + 0 * 3 + zp] + beta[s * 3 + 0];
    double t1 = ltm[s * 9 + 1 * 3 + zp] + beta[s * 3 + 1];
    double t2 = ltm[s * 9 + 2 * 3 + zp] + beta[s * 3 + 2];
    double mx = t0;
    if (t1 > mx) mx = t1;
    if (t2 > mx) mx = t2;
    double sm = d_exp(t0 - mx) + d_exp(t1 - mx) + d_exp(t2 - mx);
    return d_log(sm) + mx;
}

// Forward filter / backward sample of Z (Update_Z_subtree, bpp_c.cpp:1182-1293).
// Z filter of the FP32-partial path: linear FP64 values normalised per node
// (the log-space filter below needs three exp and a log per message; here one
// exp per node and state).  Transition matrix T[zc][zp] from g, l, l2
// (bpp_c.cpp:573-599); fixed nodes cannot be in state 2.  Draws use the same
// stream words as the log-space filter.
// Inverse-CDF draw over three FP32 weights from one 32-bit word (24-bit
// uniform), as the FP32 path's internal-base draws take theirs.
__device__ __forceinline__ int categorical3f(const float* p, uint32_t wd) {
    const float u = ((float)(wd >> 8) + 0.5f) * 5.9604644775390625e-08f;
    const float c0 = p[0], c1 = c0 + p[1], c2 = c1 + p[2];
    const float t = u * c2;
    if (t < c2) return (t >= c0) + (t >= c1);
    for (int k = 2; k >= 0; k--)
        if (p[k] > 0) return k;
    return 3;
}

// The Z filter of the FP32 path in linear FP32: the emissions, relative to
// each node's largest, as FP32 weights; messages up the tree with exact
// power-of-two normalisation; draws from the same stream positions as the
// FP64 filter, with FP32 categoricals.
template <typename Real>
__device__ int update_z_linear(Ctx<Real>& c, uint64_t pos) {
    const int T = c.T, m = c.cs->m;
    const float gr = (float)c.trd[TR_G * T + m], lr = (float)c.trd[TR_L * T + m], lr2 = (float)c.trd[TR_L2 * T + m];
    float* beta = (float*)c.beta;   // [N][3] in the FP64 buffer's space
    for (int i = threadIdx.x; i < c.n_nodes; i += blockDim.x) {
        const int s = c.nodes[i];
        const double e0 = c.emis[s * 3 + 0], e1 = c.emis[s * 3 + 1], e2 = c.emis[s * 3 + 2];
        const bool ban = c.fixZ[s] == 1;
        double mx = e0 > e1 ? e0 : e1;
        if (!ban && e2 > mx) mx = e2;
        beta[s * 3 + 0] = expf((float)(e0 - mx));
        beta[s * 3 + 1] = expf((float)(e1 - mx));
        beta[s * 3 + 2] = ban ? 0.0f : expf((float)(e2 - mx));
        c.changed[s] = 0;
    }
    __syncthreads();
    // the tree's levels on one warp (warp barriers between levels); the
    // message of child ci to parent state zp is sum_zc T[zc][zp] beta_ci[zc]
    // with T the fixed nodes' (no state 2) or the free nodes' matrix
    int err = 0;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        for (int h = 0; h < c.n_hlev; h++) {
            const int a = c.hlev_start[h], b = c.hlev_start[h + 1];
            for (int i = a + lane; i < b; i += 32) {
                const int p = c.hlev_nodes[i];
                float v0 = beta[p * 3 + 0], v1 = beta[p * 3 + 1], v2 = beta[p * 3 + 2];
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const int ci = q ? c.c2b[p] : c.c2a[p];
                    const float b0 = beta[ci * 3 + 0], b1 = beta[ci * 3 + 1], b2 = beta[ci * 3 + 2];
                    const bool fx = c.fixZ[ci] == 1;
                    v0 *= fmaf(gr, b1, (1 - gr) * b0);
                    v1 *= fx ? b1 : fmaf(lr, b2, (1 - lr) * b1);
                    v2 *= fx ? 0.0f : fmaf(1 - lr2, b2, lr2 * b1);
                }
                // exact power-of-two normalisation (the values are relative)
                const float mx = fmaxf(v0, fmaxf(v1, v2));
                if (mx > 0) {
                    int ex;
                    frexpf(mx, &ex);
                    v0 = ldexpf(v0, -ex); v1 = ldexpf(v1, -ex); v2 = ldexpf(v2, -ex);
                }
                beta[p * 3 + 0] = v0; beta[p * 3 + 1] = v1; beta[p * 3 + 2] = v2;
            }
            __syncwarp();
        }
        if (lane == 0) {
            const float pr[3] = {0.5f * beta[c.root * 3 + 0], 0.5f * beta[c.root * 3 + 1], 0.0f};
            uint32_t wd[4];
            philox4x32_10((uint32_t)(pos >> 2), (uint32_t)(pos >> 34), 0u, 0u, dM.seed, 0u, wd);
            int nn = categorical3f(pr, wd[pos & 3]);
            if (nn > 2) { err = 1; nn = c.Z[c.root]; }
            if (nn != c.Z[c.root]) c.changed[c.root] = 1;
            c.Z[c.root] = (int8_t)nn;
        }
        __syncwarp();
        for (int d = 0; d < c.n_dlev; d++) {
            const int a = c.dlev_start[d], b = c.dlev_start[d + 1];
            for (int i = a + lane; i < b; i += 32) {
                const int s = c.dlev_nodes[i];
                const int zp = c.Z[c.par[s]];
                const bool fx = c.fixZ[s] == 1;
                const float b0 = beta[s * 3 + 0], b1 = beta[s * 3 + 1], b2 = beta[s * 3 + 2];
                float pr[3];
                if (zp == 0) { pr[0] = (1 - gr) * b0; pr[1] = gr * b1; pr[2] = 0.0f; }
                else if (zp == 1) { pr[0] = 0.0f; pr[1] = fx ? b1 : (1 - lr) * b1; pr[2] = fx ? 0.0f : lr * b2; }
                else { pr[0] = 0.0f; pr[1] = fx ? 0.0f : lr2 * b1; pr[2] = fx ? 0.0f : (1 - lr2) * b2; }
                const uint64_t w = pos + 1 + (uint64_t)(c.n_nodes - 2 - c.pos[s]);
                uint32_t wd[4];
                philox4x32_10((uint32_t)(w >> 2), (uint32_t)(w >> 34), 0u, 0u, dM.seed, 0u, wd);
                int nn = categorical3f(pr, wd[w & 3]);
                if (nn > 2) { err = 1; nn = c.Z[s]; }
                if (nn != c.Z[s]) c.changed[s] = 1;
                c.Z[s] = (int8_t)nn;
            }
            __syncwarp();
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) c.local.z_draws += c.n_nodes;
    return err;
}

template <typename Real>
__device__ int update_z(Ctx<Real>& c, uint64_t pos) {
    if (sizeof(Real) == 4) return update_z_linear(c, pos);
    const double NI = -CUDART_INF;
    for (int i = threadIdx.x; i < c.n_nodes; i += blockDim.x) {
        int s = c.nodes[i];
        for (int k = 0; k < 3; k++) c.beta[s * 3 + k] = c.emis[s * 3 + k];
        if (c.fixZ[s] == 1) c.beta[s * 3 + 2] = NI;
        c.changed[s] = 0;
    }
    __syncthreads();
    // the tree's levels on one warp (warp barriers between levels)
    int err = 0;
    if (threadIdx.x >= 32) goto done;
    for (int h = 0; h < c.n_hlev; h++) {
        int a = c.hlev_start[h], b = c.hlev_start[h + 1];
        for (int i = a * 3 + (int)threadIdx.x; i < b * 3; i += 32) {
            int p = c.hlev_nodes[i / 3];
            int zp = i % 3;
            double v = c.beta[p * 3 + zp];
            v += msg(c.ltm, c.beta, c.c2a[p], zp);
            v += msg(c.ltm, c.beta, c.c2b[p], zp);
            c.beta[p * 3 + zp] = v;
        }
        __syncwarp();
    }
    if (threadIdx.x == 0) {
        const double prior_z[3] = {d_log(0.5), d_log(0.5), NI};
        double lp[3], pr[3];
        for (int k = 0; k < 3; k++) lp[k] = c.beta[c.root * 3 + k] + prior_z[k];
        double mx = lp[0];
        if (lp[1] > mx) mx = lp[1];
        if (lp[2] > mx) mx = lp[2];
        for (int k = 0; k < 3; k++) pr[k] = d_exp(lp[k] - mx);
        uint32_t wd[4];
        philox4x32_10((uint32_t)(pos >> 2), (uint32_t)(pos >> 34), 0u, 0u, dM.seed, 0u, wd);
        int nn = categorical(3, pr, word_to_uniform(wd[pos & 3]));
        if (nn > 2) { err = 1; nn = c.Z[c.root]; }
        if (nn != c.Z[c.root]) c.changed[c.root] = 1;
        c.Z[c.root] = (int8_t)nn;
    }
    __syncwarp();
    for (int d = 0; d < c.n_dlev; d++) {
        int a = c.dlev_start[d], b = c.dlev_start[d + 1];
        for (int i = a + (int)threadIdx.x; i < b; i += 32) {
            int s = c.dlev_nodes[i];
            int zp = c.Z[c.par[s]];
            double lt[3], pr[3];
            for (int k = 0; k < 3; k++) lt[k] = c.ltm[s * 9 + k * 3 + zp] + c.beta[s * 3 + k];
            double mx = lt[0];
            if (lt[1] > mx) mx = lt[1];
            if (lt[2] > mx) mx = lt[2];
            for (int k = 0; k < 3; k++) pr[k] = d_exp(lt[k] - mx);
            uint64_t w = pos + 1 + (uint64_t)(c.n_nodes - 2 - c.pos[s]);
            uint32_t wd[4];
            philox4x32_10((uint32_t)(w >> 2), (uint32_t)(w >> 34), 0u, 0u, dM.seed, 0u, wd);
            int nn = categorical(3, pr, word_to_uniform(wd[w & 3]));
            if (nn > 2) { err = 1; nn = c.Z[s]; }
            if (nn != c.Z[s]) c.changed[s] = 1;
            c.Z[s] = (int8_t)nn;
        }
        __syncwarp();
    }
done:
    __syncthreads();
    if (threadIdx.x == 0) c.local.z_draws += c.n_nodes;
    return err;
}

// Flags of proper ancestors of flagged nodes (getUpdateNode, bpp_c.cpp:620-642).
template <typename Real>
__device__ void mark_ancestors(Ctx<Real>& c, const int8_t* src, int8_t* dst, int mode, int* tmp) {
    // mode 0: src = changed flags; mode 1: Z == 2 (non-missing); mode 2: Z == 1 (non-missing)
    for (int i = threadIdx.x; i < c.N; i += blockDim.x) dst[i] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < c.n_nodes; i += blockDim.x) {
        int s = c.nodes[i];
        bool f;
        if (mode == 0) f = src[s];
        else f = !c.missing[s] && c.Z[s] == (mode == 1 ? 2 : 1);
        if (!f) continue;
        int j = c.par[s];
        while (j >= 0 && j < c.N) {
            dst[j] = 1;
            j = c.par[j];
        }
    }
    __syncthreads();
}

// Log density of Gamma(shape a, scale b) at x > 0 without the exp/log round
// trip: (a - 1) log x - x / b - lgamma(a) - a log b, with log x given.
__device__ __forceinline__ double lgamma_pdf_lx(double x, double lx, double a, double b, double lga_alogb) {
    return (a - 1.0) * lx - x / b - lga_alogb;
}

// One Metropolis-Hastings update of the accelerated (neut) or conserved rate
// (sample_rate, bpp_c.cpp:930-1176), M = 1, adaptive factor 0.5.
// FP64 partials follow the reference's arithmetic term by term.  FP32
// partials keep the MH ratio in FP64 but evaluate it from cached logs of the
// current rate and proposal scale (one new log per proposal, plus one lgamma
// for the accelerated rate's Gamma proposal), and draw the proposal in FP32.
template <typename Real>
__device__ double sample_rate(Ctx<Real>& c, const double* dist2, bool neut, double old_rate, int* tmp) {
    ChainScalars* cs = c.cs;
    const bool f32 = sizeof(Real) == 4;
    const int8_t* unv = neut ? c.unvN : c.unvC;
    const int cls = neut ? P_NEUT : P_CONS;
    double prior_a = neut ? dM.nprior_a : dM.cprior_a;
    double prior_b = neut ? dM.nprior_b : dM.cprior_b;
    const int m = cs->m;
    __syncthreads();
    if (!unv[c.root]) {
        // no branch in the class: draw from the prior (bpp_c.cpp:940-964)
        if (threadIdx.x == 0) {
            double cur = old_rate;
            if (cs->resZ != 0) {
                if (f32) {
                    StreamReader32 rd;
                    rd.init(dM.seed, cs->pos);
                    cur = (double)rd.gamma((float)prior_a, (float)prior_b);
                    cs->pos = rd.pos;
                } else {
                    StreamReader rd;
                    rd.init(dM.seed, cs->pos);
                    cur = rd.gamma(prior_a, prior_b);
                    cs->pos = rd.pos;
                }
                if (neut) {
                    if (dM.ropt == 1 && cur < dM.nlb) cur = old_rate;
                    else if (dM.ropt == 2 && cur < c.trd[TR_C * c.T + m]) cur = old_rate;
                } else {
                    if (dM.ropt == 1 && cur > dM.cub) cur = old_rate;
                    else if (dM.ropt == 2 && cur > c.trd[TR_N * c.T + m + 1]) cur = old_rate;
                }
            }
            cs->proposal = cur;
            if (f32 && cur != old_rate) {
                if (neut) { cs->lcur_n = d_log(cur); cs->lgn_ok = 0; }
                else cs->lcur_c = d_log(cur);
            }
        }
        __syncthreads();
        double cur = cs->proposal;
        if (cur != old_rate) build_class(c, dist2, cls, cur, true, false);
        __syncthreads();
        if (threadIdx.x == 0 && cur != old_rate) { if (neut) cs->acc_n++; else cs->acc_c++; }
        __syncthreads();
        double r = cs->proposal;
        // adaptive step below
        if (threadIdx.x == 0) cs->mh_new = r;
        __syncthreads();
    } else {
        if (threadIdx.x == 0) {
            double r, proposal;
            int skip = 0;
            double cur = old_rate;
            if (f32) {
                StreamReader32 rd;
                rd.init(dM.seed, cs->pos);
                r = word_to_uniform(rd.word_at(rd.pos++));
                if (neut) proposal = (double)rd.gamma((float)(cur / cs->prop_n), (float)cs->prop_n);
                else {
                    double ip = 1.0 / cs->prop_c;
                    proposal = cur * (r * (cs->prop_c - ip) + ip);
                }
                cs->pos = rd.pos;
            } else {
                StreamReader rd;
                rd.init(dM.seed, cs->pos);
                r = rd.uniform();
                if (neut) {
                    proposal = rd.gamma(__ddiv_rn(cur, cs->prop_n), cs->prop_n);
                } else {
                    double ip = __ddiv_rn(1.0, cs->prop_c);
                    double u = __dadd_rn(__dmul_rn(r, __dsub_rn(cs->prop_c, ip)), ip);
                    proposal = __dmul_rn(cur, u);
                }
                cs->pos = rd.pos;
            }
            if (neut) {
                if (dM.ropt == 1 && proposal < dM.nlb) skip = 1;
                else if (dM.ropt == 2 && proposal < c.trd[TR_C * c.T + m]) skip = 1;
            } else {
                if (dM.ropt == 1 && proposal > dM.cub) skip = 1;
                else if (dM.ropt == 2 && proposal > c.trd[TR_N * c.T + m + 1]) skip = 1;
            }
            if (!skip && (proposal < 1e-12 || proposal > 1e8)) skip = 1;
            cs->proposal = proposal;
            cs->skip = skip;
            cs->mh_new = r;  // keep r for the decision
            cs->accept = 0;
        }
        __syncthreads();
        if (!cs->skip) {
            build_prop(c, dist2, cls, cs->proposal);
            __syncthreads();
            double ll_new = prune(c, unv, true, cls);
            if (threadIdx.x == 0) {
                double proposal = cs->proposal, cur = old_rate, r = cs->mh_new;
                double MH;
                if (f32) {
                    const double lp = d_log(proposal);
                    if (neut) {
                        const double pn = cs->prop_n, lpn = cs->lpn, lc = cs->lcur_n;
                        const double s1 = proposal / pn, s2 = cur / pn;
                        const double lg1 = d_lgamma(s1);
                        const double lg2 = cs->lgn_ok ? cs->lgn : d_lgamma(s2);
                        MH = (ll_new - cs->loglik) + lgamma_pdf_lx(proposal, lp, prior_a, prior_b, dM.kn) -
                             lgamma_pdf_lx(cur, lc, prior_a, prior_b, dM.kn) +
                             lgamma_pdf_lx(cur, lc, s1, pn, lg1 + s1 * lpn) -
                             lgamma_pdf_lx(proposal, lp, s2, pn, lg2 + s2 * lpn);
                        if (d_log(r) < MH) {
                            cs->accept = 1;
                            cs->loglik = ll_new;
                            cs->lcur_n = lp;
                            cs->lgn = lg1;
                        } else {
                            cs->lgn = lg2;
                        }
                        cs->lgn_ok = 1;
                    } else {
                        const double lc = cs->lcur_c;
                        MH = (ll_new - cs->loglik) + lgamma_pdf_lx(proposal, lp, prior_a, prior_b, dM.kc) -
                             lgamma_pdf_lx(cur, lc, prior_a, prior_b, dM.kc) + lc - lp;
                        if (d_log(r) < MH) {
                            cs->accept = 1;
                            cs->loglik = ll_new;
                            cs->lcur_c = lp;
                        }
                    }
                } else {
                    if (neut)
                        MH = __dsub_rn(__dadd_rn(__dsub_rn(__dadd_rn(__dsub_rn(ll_new, cs->loglik),
                                                                   log_gamma_pdf(proposal, prior_a, prior_b)),
                                                         log_gamma_pdf(cur, prior_a, prior_b)),
                                               log_gamma_pdf(cur, __ddiv_rn(proposal, cs->prop_n), cs->prop_n)),
                                       log_gamma_pdf(proposal, __ddiv_rn(cur, cs->prop_n), cs->prop_n));
                    else
                        MH = __dsub_rn(__dadd_rn(__dsub_rn(__dadd_rn(__dsub_rn(ll_new, cs->loglik),
                                                                   log_gamma_pdf(proposal, prior_a, prior_b)),
                                                         log_gamma_pdf(cur, prior_a, prior_b)),
                                               d_log(cur)),
                                       d_log(proposal));
                    if (d_log(r) < MH) {
                        cs->accept = 1;
                        cs->loglik = ll_new;
                    }
                }
            }
            __syncthreads();
            if (cs->accept) {
                for (int i = threadIdx.x; i < c.n_int; i += blockDim.x) {
                    int s = c.internal[i];
                    if (unv[s] && !c.missing[s]) c.cur[s] ^= 1;
                }
                accept_class(c, dist2, cls, cs->proposal);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double cur = cs->accept ? cs->proposal : old_rate;
            if (cur != old_rate) { if (neut) cs->acc_n++; else cs->acc_c++; }
            cs->mh_new = cur;
        }
        __syncthreads();
    }
    double cur = c.cs->mh_new;
    // adaptive proposal scale (bpp_c.cpp:1145-1171)
    if (threadIdx.x == 0 && (m + 1) % dM.adapt_freq == 0) {
        int blocks = (m + 1) / dM.adapt_freq;
        double step = fmin(0.5, 1 / sqrt((double)blocks));
        double scale_adj;
        if (neut) {
            double rate = (double)cs->acc_n / dM.adapt_freq;
            if (rate > 0.44) scale_adj = d_exp(step);
            else if (rate < 0.23) scale_adj = d_exp(-step);
            else scale_adj = 1;
            cs->prop_n = __dmul_rn(cs->prop_n, scale_adj);
            if (cs->prop_n > 1) cs->prop_n = 1;
            cs->acc_n = 0;
            if (f32) { cs->lpn = d_log(cs->prop_n); cs->lgn_ok = 0; }
        } else {
            double rate = (double)cs->acc_c / dM.adapt_freq;
            if (rate > 0.44) scale_adj = d_exp(step);
            else if (rate < 0.23) scale_adj = d_exp(-step);
            else scale_adj = 1;
            cs->prop_c = d_pow(cs->prop_c, scale_adj);
            if (cs->prop_c < 1.0001) cs->prop_c = 1.0001;
            cs->acc_c = 0;
        }
    }
    __syncthreads();
    return cur;
}

// Rank selection: the element that std::sort would put at index T/2 (bpp_c2.cpp:742-755).
__device__ double median_of(const double* x, int T, double* red) {
    int target = T / 2;
    __syncthreads();
    for (int i = threadIdx.x; i < T; i += blockDim.x) {
        double v = x[i];
        int lt = 0, eqb = 0;
        for (int j = 0; j < T; j++) {
            double u = x[j];
            lt += (u < v);
            eqb += (u == v && j < i);
        }
        int r = lt + eqb;
        if (r == target) red[RED_MED] = v;
    }
    __syncthreads();
    double r = red[RED_MED];
    __syncthreads();
    return r;
}


// Prior of a Z configuration (bpp_c2.cpp:131-163): Beta-Binomial terms + root prior.
template <typename Real>
__device__ double prior_config(Ctx<Real>& c, const int8_t* z) {
    double nZ[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int k = 0; k + 1 < c.n_nodes; k++) {
        int s = c.nodes[k];
        nZ[z[s]][z[c.par[s]]] += 1;
    }
    double pz = lnbeta(dM.ga + nZ[1][0] + nZ[2][0], dM.gb + nZ[0][0]) - lnbeta(dM.ga, dM.gb);
    for (int k = 0; k + 1 < c.n_nodes; k++) {
        int s = c.nodes[k];
        if (c.fixZ[s] == 1) nZ[z[s]][z[c.par[s]]] -= 1;
    }
    pz += lnbeta(dM.la + nZ[2][1], dM.lb + nZ[1][1]) - lnbeta(dM.la, dM.lb);
    if (dM.l2a > 0) pz += lnbeta(dM.l2a + nZ[1][2], dM.l2b + nZ[2][2]) - lnbeta(dM.l2a, dM.l2b);
    pz += (z[c.root] == 2) ? -CUDART_INF : d_log(0.5);
    return pz;
}

// Marginal likelihood of one model (Eval2, bpp_c2.cpp:14-353).
template <typename Real>
__device__ double eval2(Ctx<Real>& c, const double* dist2, int resZ, int* tmp, int* n_conf_out) {
    ChainScalars* cs = c.cs;
    const int burn = c.burn, mcmc = c.mcmc, T = c.T;
    int8_t* Zm = c.maxz;  // Max_Z
    // uncertain nodes
    for (int s = threadIdx.x; s < c.N; s += blockDim.x) {
        int cnt = 0;
        for (int i = burn; i < T; i++) cnt += (c.trz[(size_t)i * c.N + s] == Zm[s]);
        c.changed[s] = cnt < mcmc;   // reuse: uncertain flag
    }
    __syncthreads();
    // hashes of the uncertain projection
    for (int i = burn + threadIdx.x; i < T + 1; i += blockDim.x) {
        const int8_t* z = (i < T) ? c.trz + (size_t)i * c.N : Zm;
        uint64_t h = 0xcbf29ce484222325ull;
        for (int s = 0; s < c.N; s++)
            if (c.changed[s]) h = fnv_step(h, (uint8_t)z[s]);
        c.hash[i - burn] = h;
    }
    __syncthreads();
    auto same = [&](const int8_t* a, const int8_t* b) {
        for (int s = 0; s < c.N; s++)
            if (c.changed[s] && a[s] != b[s]) return false;
        return true;
    };
    // rep[i]: largest index >= i with the same projection; cfg[i] = -2 if it equals Max_Z's
    for (int i = burn + threadIdx.x; i < T; i += blockDim.x) {
        const int8_t* zi = c.trz + (size_t)i * c.N;
        uint64_t hi = c.hash[i - burn];
        int r = i;
        for (int j = T - 1; j > i; j--) {
            if (c.hash[j - burn] == hi && same(c.trz + (size_t)j * c.N, zi)) { r = j; break; }
        }
        c.rep[i - burn] = r;
        c.cfg[i - burn] = (hi == c.hash[T - burn] && same(zi, Zm)) ? -2 : -1;
    }
    __syncthreads();
    // configuration ids in first-occurrence order scanning from the last sample (bpp_c2.cpp:65-116)
    if (threadIdx.x == 0) {
        int nconf = 1;
        c.first[0] = -1;   // Max_Z
        c.head[0] = -1;
        for (int i = T - 1; i >= burn; i--) {
            int k = i - burn;
            int j;
            if (c.cfg[k] == -2) j = 0;
            else if (c.rep[k] == i) { j = nconf++; c.first[j] = i; c.head[j] = -1; }
            else j = c.cfg[c.rep[k] - burn];
            c.cfg[k] = j;
        }
        // members of each config in decreasing sample index: build lists
        for (int j = 0; j < nconf; j++) c.head[j] = -1;
        for (int i = burn; i < T; i++) {     // prepend in increasing order -> list in decreasing order
            int k = i - burn;
            int j = c.cfg[k];
            c.nxt[k] = c.head[j];
            c.head[j] = k;
        }
        cs->n_conf = nconf;
    }
    __syncthreads();
    const int nconf = cs->n_conf;
    *n_conf_out = nconf;
    // per-config sums in the reference's order (bpp_c2.cpp:105-113)
    double* CNT = c.cstat;
    double* VC = CNT + (mcmc + 2);
    double* MC = VC + (mcmc + 2);
    double* VN = MC + (mcmc + 2);
    double* MN = VN + (mcmc + 2);
    double* CV = MN + (mcmc + 2);
    double* SF = CV + (mcmc + 2);
    double* LD = SF + (mcmc + 2);
    double* PZ = LD + (mcmc + 2);
    const double* trN = c.trd + TR_N * T;
    const double* trC = c.trd + TR_C * T;
    const double* trF = c.trd + TR_FULL * T;
    for (int j = threadIdx.x; j < nconf; j += blockDim.x) {
        double n = 0, vc = 0, mc = 0, vn = 0, mn = 0, cv = 0, sf = 0;
        for (int k = c.head[j]; k >= 0; k = c.nxt[k]) {
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
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nconf; j += blockDim.x) {
        double w = CNT[j] / mcmc;
        LD[j] = 0;
        if (w < 0.02) continue;
        const int8_t* z = (j == 0) ? Zm : c.trz + (size_t)c.first[j] * c.N;
        double pz = prior_config(c, z);
        PZ[j] = pz;
        SF[j] = __dadd_rn(SF[j], __ddiv_rn(__dmul_rn(CNT[j], pz), (double)mcmc));
        double nj = CNT[j];
        double ld;
        if (resZ == 0) {
            ld = __dsub_rn(d_log(__dsub_rn(VC[j], __ddiv_rn(__dmul_rn(MC[j], MC[j]), nj))), d_log(nj));
        } else {
            double vc = __dsub_rn(VC[j], __ddiv_rn(__dmul_rn(MC[j], MC[j]), nj));
            double vn = __dsub_rn(VN[j], __ddiv_rn(__dmul_rn(MN[j], MN[j]), nj));
            double cov = __dsub_rn(CV[j], __ddiv_rn(__dmul_rn(MN[j], MC[j]), nj));
            ld = __dsub_rn(d_log(__dsub_rn(__dmul_rn(vc, vn), __dmul_rn(cov, cov))), __dmul_rn(2.0, d_log(nj)));
        }
        LD[j] = ld;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double VB = 0;
        int eff = 0;
        for (int j = 0; j < nconf; j++) {
            double w = CNT[j] / mcmc;
            if (w < 0.02) continue;
            if (isnan(LD[j])) continue;
            eff += (int)CNT[j];
            VB = __dsub_rn(VB, __dmul_rn(w, d_log(CNT[j])));
            VB = __dadd_rn(VB, SF[j]);
            VB = __dadd_rn(VB, __ddiv_rn(__dmul_rn(__dmul_rn(0.5, LD[j]), CNT[j]), (double)mcmc));
        }
        cs->eff = eff;
        cs->vb = VB;
    }
    __syncthreads();
    double VB = cs->vb;
    if (cs->eff == 0) {
        // no dominant configuration: q(r, Z) = q(r) q(Z) at the mean rates (bpp_c2.cpp:199-316)
        double varn = 0, varc = 0, cov = 0, meann = 0, meanc = 0;
        for (int j = 0; j < nconf; j++) {
            varc = __dadd_rn(varc, VC[j]);
            meanc = __dadd_rn(meanc, MC[j]);
            if (resZ != 0) { meann = __dadd_rn(meann, MN[j]); varn = __dadd_rn(varn, VN[j]); cov = __dadd_rn(cov, CV[j]); }
        }
        double rn = meann / mcmc, rc = meanc / mcmc;
        build_class(c, dist2, P_CONS, rc, true, true);
        if (resZ != 0) build_class(c, dist2, P_NEUT, rn, true, true);
        __syncthreads();
        // one likelihood per configuration.  After the first (a full pass),
        // only the proper ancestors of branches whose class changed since the
        // previous configuration are pruned again: a node's partial depends
        // on its children's classes alone, so every partial, and the
        // likelihood, is that of a full pass.  When only the root's class
        // changed no partial changes and the likelihood is the previous one.
        double ll = 0;
        for (int j = 0; j < nconf; j++) {
            const int8_t* z = (j == 0) ? Zm : c.trz + (size_t)c.first[j] * c.N;
            for (int s = threadIdx.x; s < c.N; s += blockDim.x) {
                c.unvN[s] = (j == 0) || (c.Z[s] != z[s]);   // free after the chain
                c.Z[s] = z[s];
                if (j == 0) {
                    c.unv[s] = 1;
                    c.cur[s] = 0;
                }
            }
            __syncthreads();
            if (j > 0) mark_ancestors(c, c.unvN, c.unv, 0, tmp);
            double pz = prior_config(c, z);
            if (c.unv[c.root]) ll = prune(c, c.unv, false, -1);
            if (threadIdx.x == 0) SF[j] = __dadd_rn(ll, pz);
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            double mx = SF[0];
            for (int j = 1; j < nconf; j++) if (SF[j] > mx) mx = SF[j];
            double v;
            if (mx == -CUDART_INF) v = -CUDART_INF;
            else {
                double sm = 0;
                for (int j = 0; j < nconf; j++) sm += d_exp(SF[j] - mx);
                v = d_log(sm) + mx;
            }
            v += log_gamma_pdf(rc, dM.cprior_a, dM.cprior_b);
            if (resZ != 0) v += log_gamma_pdf(rn, dM.nprior_a, dM.nprior_b);
            double logdet;
            if (resZ == 0) {
                varc -= meanc * meanc / mcmc;
                logdet = d_log(varc) - d_log((double)mcmc);
                v += 0.5 * logdet + 0.5 * d_log(2 * CUDART_PI);
            } else {
                varn -= meann * meann / mcmc;
                varc -= meanc * meanc / mcmc;
                cov -= meann * meanc / mcmc;
                logdet = d_log(varc * varn - cov * cov) - 2 * d_log((double)mcmc);
                v += 0.5 * logdet + d_log(2 * CUDART_PI);
            }
            cs->vb = v;
        }
        __syncthreads();
        VB = cs->vb;
    } else {
        double f = (double)mcmc / cs->eff;
        if (resZ != 0) VB = VB * f + d_log((double)mcmc) + d_log(2 * CUDART_PI) + 1;
        else VB = VB * f + d_log((double)mcmc) + 0.5 * (d_log(2 * CUDART_PI) + 1);
    }
    __syncthreads();
    return VB;
}

// ---------------------------------------------------------------------------
// The chain kernel
// ---------------------------------------------------------------------------
// FP32 runs 256 threads with two blocks per SM (128 registers a thread);
// FP64 runs 128 threads and may use more registers.
// Shared-memory pointers of a chain context (layout SmemLayout).
template <typename Real>
__device__ void bind_smem(Ctx<Real>& c, unsigned char* smem, int N, int BT, int D) {
    SmemLayout<Real> L = SmemLayout<Real>::make(N, BT, D);
    TopoLayout TL = TopoLayout::make(N);
    c.N = N;
    c.D = D;
    c.ptd = (sizeof(Real) == 8) ? (double*)(smem + L.ptd) : nullptr;
    c.ptr = (sizeof(Real) == 8) ? (Real*)(smem + L.ptd) : (Real*)(smem + L.ptr_);
    c.ltm = (double*)(smem + L.ltm);
    c.emis = (double*)(smem + L.emis);
    c.beta = (double*)(smem + L.beta);
    c.cnt = (unsigned*)(smem + L.cnt);
    c.red = (double*)(smem + L.red);
    int16_t* t16 = (int16_t*)(smem + L.i16);
    c.nodes = t16 + TL.nodes; c.internal = t16 + TL.internal; c.c2a = t16 + TL.c2a; c.c2b = t16 + TL.c2b;
    c.par = t16 + TL.par; c.irank = t16 + TL.irank; c.pos = t16 + TL.pos; c.missing = t16 + TL.missing;
    c.upc = t16 + TL.upc; c.upcc = t16 + TL.upcc; c.hlev_start = t16 + TL.hlev_start;
    c.hlev_nodes = t16 + TL.hlev_nodes; c.dlev_start = t16 + TL.dlev_start; c.dlev_nodes = t16 + TL.dlev_nodes;
    c.sord = t16 + TL.sord; c.sflag = t16 + TL.sflag;
    int8_t* t8 = (int8_t*)(smem + L.i8);
    c.Z = t8; c.fixZ = t8 + N; c.changed = t8 + 2 * N; c.unv = t8 + 3 * N; c.unvN = t8 + 4 * N;
    c.unvC = t8 + 5 * N; c.cur = t8 + 6 * N; c.maxz = t8 + 7 * N;
    c.bases = (int8_t*)(smem + L.scr);
    c.ring = (Real*)(smem + L.ring);
    c.stk = (Real*)(smem + L.scr);
    c.stks = (int32_t*)(smem + L.stks);
    c.pn = (PNode*)(smem + L.desc);
    c.sn = (SNode*)(smem + L.desc);
}

// Register budgets (launch bounds MAXT threads, MINB blocks per SM): FP32
// partials come in three (128 registers: four 128-thread chains per SM; 168:
// three; 255: two, or one of 256 threads), chosen per taxon count by the
// host's trial-launch tuner; FP64 partials use one (255).
template <typename Real, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) chain_kernel(ChainParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ ChainScalars cs_;
    __shared__ int tmp_;
    __shared__ int elem_;
    const int N = dM.N, S = dM.S;
    const int BT = blockDim.x;
    TopoLayout TL = TopoLayout::make(N);
    Ctx<Real> c;
    c.S = S;
    bind_smem(c, smem, N, BT, P.stack_cap);
    int16_t* t16 = c.nodes;
    double* dist2_ = (double*)(smem + SmemLayout<Real>::make(N, BT, P.stack_cap).dist);
    c.cs = &cs_;
    c.burn = P.trial_mcmc > 0 ? P.trial_burn : dM.burnin;
    c.mcmc = P.trial_mcmc > 0 ? P.trial_mcmc : dM.mcmc;
    c.T = c.burn + c.mcmc;
    const int T = c.T;
    char* ws = P.ws + (size_t)blockIdx.x * P.ws_stride;
    WsLayout W = WsLayout::make(P.n_int_max, P.GGp_max, T, c.mcmc, N, sizeof(Real));
    c.lam = (Real*)(ws + W.lam);
    c.scl = (int32_t*)(ws + W.scale);
    c.act = (int8_t*)(ws + W.tg);
    c.trz = (int8_t*)(ws + W.trz);
    c.trd = (double*)(ws + W.trd);
    c.hash = (uint64_t*)(ws + W.hash);
    c.rep = (int32_t*)(ws + W.rep);
    c.cfg = (int32_t*)(ws + W.cfg);
    c.nxt = (int32_t*)(ws + W.nxt);
    c.head = (int32_t*)(ws + W.head);
    c.first = (int32_t*)(ws + W.first);
    c.cstat = (double*)(ws + W.cstat);
    const int TI = dM.trace_iters < T ? dM.trace_iters : T;

    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            if (!P.stream) {
                const int i = atomicAdd(P.next_elem, 1);
                elem_ = (i < P.n_elem && P.order) ? P.order[i] : i;
            } else {
                // take the next published queue position; return when the host
                // asks the idle blocks to stop (q_stop), or after idle_ns
                // without work at the latest (the host launches again when needed)
                elem_ = P.n_elem;
                const unsigned long long t0 = globaltimer_ns();
                for (;;) {
                    const int h = *(volatile int*)P.q_head;
                    const int t = *P.q_tail;
                    if (h >= t && *P.q_stop) break;
                    if (h < t) {
                        if (atomicCAS(P.q_head, h, h + 1) == h) {
                            __threadfence_system();   // the slot id and its data after the tail
                            elem_ = P.q_slot[h % P.q_cap];
                            break;
                        }
                        continue;
                    }
                    if ((long long)(globaltimer_ns() - t0) > P.idle_ns) {
                        if (P.counters) atomicAdd(&P.counters->idle_exits, 1ull);
                        break;
                    }
                    __nanosleep(4000);
                }
            }
        }
        __syncthreads();
        const int e = elem_;
        if (e < 0 || e >= P.n_elem) break;
        long long t_start = clock64();
        ElemHeader H;
        if (P.stream) {
            // the host rewrote this slot while the kernel ran: read it past L1
            const int* src = (const int*)(P.hdr + e);
            int* dst = (int*)&H;
            for (int i = 0; i < (int)(sizeof(ElemHeader) / 4); i++) dst[i] = __ldcg(src + i);
        } else {
            H = P.hdr[e];
        }
        DevResult* R = P.results + e;
        if (H.filtered) {
            if (threadIdx.x == 0) R->status = 1;
            continue;
        }
        c.local = DevCounters{};
        c.GG = H.GG; c.GGp = H.GGp; c.root = H.root; c.n_nodes = H.n_nodes; c.n_int = H.n_int;
        c.n_hlev = H.n_hlev; c.n_dlev = H.n_dlev; c.tg_draws = H.tg_draws;
        c.codes = P.blob + H.codes_off;
        c.prefix = (const int32_t*)(P.blob + H.prefix_off);
        const int16_t* topo = (const int16_t*)(P.blob + H.topo_off);
        const double* d2 = (const double*)(P.blob + H.topo_off + (size_t)((TL.total * 2 + 15) & ~15));
        const int8_t* tg0 = (const int8_t*)(P.blob + H.tg_off);
        if (!P.stream) {
            for (int i = threadIdx.x; i < TL.total; i += BT) t16[i] = topo[i];
            for (int i = threadIdx.x; i < N; i += BT) dist2_[i] = d2[i];
            for (size_t i = threadIdx.x; i < (size_t)c.n_int * c.GGp; i += BT) c.act[i] = tg0[i];
        } else {
            // element data of a queue slot: copied past L1 into shared memory
            // and this CTA's workspace, which the chain then reads
            for (int i = threadIdx.x; i < TL.total; i += BT) t16[i] = __ldcg(topo + i);
            for (int i = threadIdx.x; i < N; i += BT) dist2_[i] = __ldcg(d2 + i);
            for (size_t i = threadIdx.x; i < (size_t)c.n_int * c.GGp; i += BT) c.act[i] = __ldcg(tg0 + i);
            const int nw = (int)(((size_t)S * c.GGp) / 4);
            const int* csrc = (const int*)c.codes;
            int* cdst = (int*)(ws + W.codes);
            for (int i = threadIdx.x; i < nw; i += BT) cdst[i] = __ldcg(csrc + i);
            for (int i = threadIdx.x; i <= c.GG; i += BT) ((int32_t*)(ws + W.prefix))[i] = __ldcg(c.prefix + i);
            c.codes = (const uint8_t*)(ws + W.codes);
            c.prefix = (const int32_t*)(ws + W.prefix);
        }
        if (threadIdx.x == 0) {
            cs_.pos = 0;
            cs_.acc_n = 0;
            cs_.acc_c = 0;
            cs_.status = 0;
        }
        for (int i = threadIdx.x; i < N; i += BT) c.maxz[i] = 0;
        __syncthreads();
        const int resZ_of[3] = {0, 2, 1};
        for (int mi = P.first_model; mi < 3; mi++) {
            const int resZ = resZ_of[mi];
            // ---------------- initMCMC (bpp_c.cpp:131-343) ----------------
            if (threadIdx.x == 0) {
                cs_.resZ = resZ;
                cs_.mi = mi;
                cs_.prop_c = 1.2;
                cs_.prop_n = (double)1 / c.GG * 10;
                cs_.maxll = -CUDART_INF;
                cs_.max_m = 0;
                c.trd[TR_N * T + 0] = dM.init_n;
                c.trd[TR_C * T + 0] = dM.init_c;
                c.trd[TR_L * T + 0] = dM.init_l;
                c.trd[TR_L2 * T + 0] = (dM.l2a == 0) ? 0.0 : dM.init_l2;
                c.trd[TR_G * T + 0] = dM.init_g;
                if (P.start_rates) {
                    // SAMPLE_HYPER: the rates the previous chain stopped at (bpp_c.cpp:165-177)
                    const double* sr = P.start_rates + (size_t)e * 5;
                    c.trd[TR_N * T + 0] = sr[0];
                    c.trd[TR_C * T + 0] = sr[1];
                    c.trd[TR_G * T + 0] = sr[2];
                    c.trd[TR_L * T + 0] = sr[3];
                    c.trd[TR_L2 * T + 0] = sr[4];
                }
                cs_.rate_n = c.trd[TR_N * T + 0];
                cs_.rate_c = c.trd[TR_C * T + 0];
                if (sizeof(Real) == 4) {
                    cs_.lcur_n = d_log(cs_.rate_n);
                    cs_.lcur_c = d_log(cs_.rate_c);
                    cs_.lpn = d_log(cs_.prop_n);
                    cs_.lgn_ok = 0;
                }
            }
            for (int i = threadIdx.x; i < N; i += BT) { c.Z[i] = -1; c.fixZ[i] = -1; c.cur[i] = 0; }
            __syncthreads();
            for (int i = threadIdx.x; i < c.n_nodes; i += BT) {
                int s = c.nodes[i];
                c.Z[s] = (s == c.root) ? 0 : 1;
                if (c.upc[s]) c.fixZ[s] = 1;
                if (s == c.root) c.fixZ[s] = 1;
                if (resZ == 2 && c.upcc[s]) c.fixZ[s] = 1;
                if (resZ == 0 && s != c.root) c.fixZ[s] = 1;
            }
            __syncthreads();
            if (P.z_start_zero) {
                // a later chain starts from bpp.cur_Z, the zero vector unless
                // SAMPLE_HYPER updates it (bpp_c.cpp:148-151, bpp.cpp:201)
                for (int i = threadIdx.x; i < N; i += BT) c.Z[i] = 0;
                __syncthreads();
            }
            if (P.start_z && P.start_z[(size_t)e * N] != -128) {
                // SAMPLE_HYPER: the Z the previous chain stopped at (bpp_c.cpp:150)
                for (int i = threadIdx.x; i < N; i += BT) c.Z[i] = P.start_z[(size_t)e * N + i];
                __syncthreads();
            }
            build_class(c, dist2_, P_NULL, 1.0, false, false);
            build_class(c, dist2_, P_NEUT, c.trd[TR_N * T + 0], true, false);
            build_class(c, dist2_, P_CONS, c.trd[TR_C * T + 0], true, false);
            __syncthreads();
            build_ltm(c, c.trd[TR_G * T], c.trd[TR_L * T], c.trd[TR_L2 * T], true);
            for (int i = threadIdx.x; i < N; i += BT) {
                c.emis[i * 3 + 0] = 0; c.emis[i * 3 + 1] = 0; c.emis[i * 3 + 2] = 0;
                if (c.missing[i]) { c.emis[i * 3 + 1] = d_log(dM.cons_to_mis); }
                c.unv[i] = 1;
            }
            __syncthreads();
            // ---------------- Gibbs (bpp_c.cpp:346-519) ----------------
            double ll0 = prune(c, c.unv, false, -1);
            if (threadIdx.x == 0) cs_.loglik = ll0;
            __syncthreads();
            long long tph = clock64();   // phase timer (thread 0): cycles per phase into the counters
#define CHAIN_PHASE(i)                                          \
    do {                                                     \
        if (threadIdx.x == 0) {                              \
            const long long t_ = clock64();                  \
            c.local.phase_cycles[i] += (unsigned long long)(t_ - tph); \
            tph = t_;                                        \
        }                                                    \
    } while (0)
            for (int m = 0; m < T; m++) {
                // MonitorChain (bpp_c.cpp:741-834)
                for (int i = threadIdx.x; i < N; i += BT) c.trz[(size_t)m * N + i] = c.Z[i];
                if (threadIdx.x == 0) {
                    cs_.m = m;
                    double ll = cs_.loglik;
                    double full = ll + 0.0;
                    if (sizeof(Real) == 4) {
                        // the rates' log priors from the logs kept with them
                        full += lgamma_pdf_lx(c.trd[TR_C * T + m], cs_.lcur_c, dM.cprior_a, dM.cprior_b, dM.kc);
                        if (resZ != 0)
                            full += lgamma_pdf_lx(c.trd[TR_N * T + m], cs_.lcur_n, dM.nprior_a, dM.nprior_b, dM.kn);
                    } else {
                        full += log_gamma_pdf(c.trd[TR_C * T + m], dM.cprior_a, dM.cprior_b);
                        if (resZ != 0) full += log_gamma_pdf(c.trd[TR_N * T + m], dM.nprior_a, dM.nprior_b);
                    }
                    c.trd[TR_LL * T + m] = ll;
                    c.trd[TR_FULL * T + m] = full;
                    tmp_ = (m >= c.burn && full > cs_.maxll) ? 1 : 0;
                    if (tmp_) { cs_.maxll = full; cs_.max_m = m; }
                }
                __syncthreads();
                if (tmp_)
                    for (int i = threadIdx.x; i < N; i += BT) c.maxz[i] = c.Z[i];
                if (m == T - 1) break;
                CHAIN_PHASE(0);
                // internal bases
                uint64_t pos = cs_.pos;
                int err = sample_emit(c, pos);
                CHAIN_PHASE(1);
                if (threadIdx.x == 0) cs_.pos = pos + (uint64_t)c.tg_draws;
                if (err) atomicOr(&cs_.status, 1);
                // latent states
                emission(c);
                CHAIN_PHASE(2);
                pos = cs_.pos;
                int zerr = update_z(c, pos);
                if (threadIdx.x == 0) cs_.pos = pos + (uint64_t)c.n_nodes;
                if (zerr) atomicOr(&cs_.status, 1);
                __syncthreads();
                CHAIN_PHASE(3);
                // partial re-prune of ancestors of changed branches (bpp_c.cpp:419-431)
                mark_ancestors(c, c.changed, c.unv, 0, &tmp_);
                int any_unv = block_or(c.unv[c.root], &tmp_);
                if (any_unv) {
                    double ll = prune(c, c.unv, false, -1);
                    if (threadIdx.x == 0) cs_.loglik = ll;
                }
                __syncthreads();
                CHAIN_PHASE(4);
                // rates (bpp_c.cpp:434-452)
                mark_ancestors(c, nullptr, c.unvN, 1, &tmp_);
                mark_ancestors(c, nullptr, c.unvC, 2, &tmp_);
                // accelerated, then conserved rate: one copy of the MH code
                // (and its prune) serves both
#pragma unroll 1
                for (int q = 0; q < 2; q++) {
                    const int row = q == 0 ? TR_N : TR_C;
                    const double rr = sample_rate(c, dist2_, q == 0, c.trd[row * T + m], &tmp_);
                    if (threadIdx.x == 0) c.trd[row * T + m + 1] = rr;
                    __syncthreads();
                    if (q == 0) CHAIN_PHASE(5);
                    else CHAIN_PHASE(6);
                }
                // transitions of Z (sample_transition, bpp_c.cpp:522-613): the
                // (child, parent) state counts in parallel (exact integers),
                // then the three Beta draws on one thread
                int* zcount = (int*)c.cnt;   // free until the next sampling pass
                if (threadIdx.x < 18) zcount[threadIdx.x] = 0;
                __syncthreads();
                for (int k = threadIdx.x; k + 1 < c.n_nodes; k += BT) {
                    const int s = c.nodes[k];
                    const int b = c.Z[s] * 3 + c.Z[c.par[s]];
                    atomicAdd(&zcount[b], 1);
                    if (c.fixZ[s] == 1) atomicAdd(&zcount[9 + b], 1);
                }
                __syncthreads();
                if (threadIdx.x == 0) {
                    double nZ[3][3];
                    for (int a = 0; a < 3; a++)
                        for (int b = 0; b < 3; b++) nZ[a][b] = (double)zcount[a * 3 + b];
                    double gr, lr, lr2;
                    if (sizeof(Real) == 4) {
                        // FP32 draws (the transition rates feed the Z filter)
                        StreamReader32 rd;
                        rd.init(dM.seed, cs_.pos);
                        gr = (double)rd.beta((float)(dM.ga + nZ[1][0] + nZ[2][0]), (float)(dM.gb + nZ[0][0]));
                        for (int a = 0; a < 3; a++)
                            for (int b = 0; b < 3; b++) nZ[a][b] -= (double)zcount[9 + a * 3 + b];
                        lr = (double)rd.beta((float)(dM.la + nZ[2][1]), (float)(dM.lb + nZ[1][1]));
                        lr2 = (dM.l2a == 0) ? 0.0 : (double)rd.beta((float)(dM.l2a + nZ[1][2]), (float)(dM.l2b + nZ[2][2]));
                        cs_.pos = rd.pos;
                    } else {
                        StreamReader rd;
                        rd.init(dM.seed, cs_.pos);
                        gr = rd.beta(dM.ga + nZ[1][0] + nZ[2][0], dM.gb + nZ[0][0]);
                        for (int a = 0; a < 3; a++)
                            for (int b = 0; b < 3; b++) nZ[a][b] -= (double)zcount[9 + a * 3 + b];
                        lr = rd.beta(dM.la + nZ[2][1], dM.lb + nZ[1][1]);
                        lr2 = (dM.l2a == 0) ? 0.0 : rd.beta(dM.l2a + nZ[1][2], dM.l2b + nZ[2][2]);
                        cs_.pos = rd.pos;
                    }
                    c.trd[TR_G * T + m + 1] = gr;
                    c.trd[TR_L * T + m + 1] = lr;
                    c.trd[TR_L2 * T + m + 1] = lr2;
                }
                __syncthreads();
                build_ltm(c, c.trd[TR_G * T + m + 1], c.trd[TR_L * T + m + 1], c.trd[TR_L2 * T + m + 1], false);
                __syncthreads();
                CHAIN_PHASE(7);
                if (threadIdx.x == 0) c.local.iters++;
            }
#undef CHAIN_PHASE
            __syncthreads();
            if (P.end_z) {
                // the state where the chain stopped (bpp_c.cpp:475-485), before
                // Eval2 reuses Z
                for (int i = threadIdx.x; i < N; i += BT) P.end_z[(size_t)e * N + i] = c.Z[i];
                if (threadIdx.x == 0) {
                    const int rws[5] = {TR_N, TR_C, TR_G, TR_L, TR_L2};
                    for (int q = 0; q < 5; q++) P.end_rates[(size_t)e * 5 + q] = c.trd[rws[q] * T + (T - 1)];
                }
                __syncthreads();
            }
            DevModelResult& MR = R->model[mi];
            if (threadIdx.x == 0) MR.max_loglik = cs_.maxll;
            // traces of the first TI iterations
            if (TI > 0 && P.tr_d) {
                double* td = P.tr_d + ((size_t)e * 3 + mi) * 6 * TI;
                const int rows[6] = {TR_LL, TR_N, TR_C, TR_G, TR_L, TR_L2};
                for (int i = threadIdx.x; i < 6 * TI; i += BT) td[i] = c.trd[rows[i / TI] * T + (i % TI)];
                int8_t* tz = P.tr_z + ((size_t)e * 3 + mi) * TI * N;
                for (int i = threadIdx.x; i < TI * N; i += BT) tz[i] = c.trz[i];
            }
            // ---------------- Eval2 ----------------
            int nconf = 0;
            double vb = eval2(c, dist2_, resZ, &tmp_, &nconf);
            // ---------------- Output_init (bpp_c2.cpp:739-785) ----------------
            double med[5];
            const int mrow[5] = {TR_N, TR_C, TR_G, TR_L, TR_L2};
            for (int q = 0; q < 5; q++) med[q] = median_of(c.trd + mrow[q] * T, T, c.red);
            if (threadIdx.x == 0) {
                MR.loglik = vb;
                for (int q = 0; q < 5; q++) MR.rates[q] = med[q];
                MR.failure = isnan(vb) ? 1 : 0;
                MR.n_configs = nconf;
                if (isnan(vb)) cs_.status |= 2;
            }
            int32_t* mz = P.max_z + ((size_t)e * 3 + mi) * N;
            for (int s = threadIdx.x; s < N; s += BT) mz[s] = c.maxz[s];
            double* pz = P.post_z + ((size_t)e * 3 + mi) * N * 4;
            for (int s = threadIdx.x; s < N; s += BT) {
                int cnt[4] = {0, 0, 0, 0};
                for (int i = c.burn; i < T; i++) {
                    int z = c.trz[(size_t)i * N + s];
                    if (z >= -1 && z <= 2) cnt[z + 1]++;
                }
                if (c.missing[s]) cnt[0] = c.mcmc;
                for (int k = 0; k < 4; k++) pz[s * 4 + k] = (double)cnt[k] / c.mcmc;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            R->status = (cs_.status & 1) ? 3 : ((cs_.status & 2) ? 2 : 0);
            R->device_ms = (double)(clock64() - t_start);
        }
        if (P.stream) {
            // publish the slot once every thread's result writes are visible
            __threadfence_system();
            __syncthreads();
            if (threadIdx.x == 0) P.done_flag[e] = 1;
        }
        // counters
        if (P.counters) {
            atomicAdd(&P.counters->edge_internal, c.local.edge_internal);
            atomicAdd(&P.counters->edge_leaf, c.local.edge_leaf);
            atomicAdd(&P.counters->tg_draws, c.local.tg_draws);
            if (threadIdx.x == 0) {
                atomicAdd(&P.counters->col_ll, c.local.col_ll);
                atomicAdd(&P.counters->z_draws, c.local.z_draws);
                atomicAdd(&P.counters->iters, c.local.iters);
                for (int q = 0; q < 8; q++) atomicAdd(&P.counters->phase_cycles[q], c.local.phase_cycles[q]);
            }
            atomicAdd(&P.counters->pmat, c.local.pmat);
        }
    }
}

// ---------------------------------------------------------------------------
// Kernel-level entry points for parity tests
// ---------------------------------------------------------------------------
__global__ void pmatrix_kernel(int n, const double* d, const double* r, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) build_pt(d[i], r[i], true, out + (size_t)i * 16);
}

__global__ void stream_kernel(uint32_t seed, uint64_t w0, int n, uint32_t* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        uint64_t w = w0 + i;
        uint32_t wd[4];
        philox4x32_10((uint32_t)(w >> 2), (uint32_t)(w >> 34), 0u, 0u, seed, 0u, wd);
        out[i] = wd[w & 3];
    }
}

// Per-column log-likelihood of one element for fixed Z and rates.
template <typename Real>
__global__ void loglik_kernel(ChainParams P, const int32_t* z, double c_rate, double n_rate, double* out) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ ChainScalars cs_;
    const int N = dM.N, S = dM.S;
    const int BT = blockDim.x;
    TopoLayout TL = TopoLayout::make(N);
    Ctx<Real> c;
    c.S = S;
    bind_smem(c, smem, N, BT, P.stack_cap);
    double* dist2_ = (double*)(smem + SmemLayout<Real>::make(N, BT, P.stack_cap).dist);
    c.cs = &cs_;
    const ElemHeader& H = P.hdr[0];
    c.GG = H.GG; c.GGp = H.GGp; c.root = H.root; c.n_nodes = H.n_nodes; c.n_int = H.n_int;
    c.codes = P.blob + H.codes_off;
    char* ws = P.ws;
    WsLayout W = WsLayout::make(P.n_int_max, P.GGp_max, 1, 1, N, sizeof(Real));
    c.lam = (Real*)(ws + W.lam);
    c.scl = (int32_t*)(ws + W.scale);
    c.act = (int8_t*)(ws + W.tg);
    c.local = DevCounters{};
    const int16_t* topo = (const int16_t*)(P.blob + H.topo_off);
    for (int i = threadIdx.x; i < TL.total; i += BT) c.nodes[i] = topo[i];
    const double* d2 = (const double*)(P.blob + H.topo_off + (size_t)((TL.total * 2 + 15) & ~15));
    for (int i = threadIdx.x; i < N; i += BT) dist2_[i] = d2[i];
    const int8_t* tg0 = (const int8_t*)(P.blob + H.tg_off);
    for (size_t i = threadIdx.x; i < (size_t)c.n_int * c.GGp; i += BT) c.act[i] = tg0[i];
    for (int i = threadIdx.x; i < N; i += BT) { c.Z[i] = (int8_t)z[i]; c.unv[i] = 1; c.cur[i] = 0; }
    if (threadIdx.x == 0) cs_.status = 0;
    __syncthreads();
    build_class(c, dist2_, P_NULL, 1.0, false, false);
    build_class(c, dist2_, P_NEUT, n_rate, true, false);
    build_class(c, dist2_, P_CONS, c_rate, true, false);
    __syncthreads();
    prune(c, c.unv, false, -1);
    __syncthreads();
    const int rir = c.irank[c.root];
    for (int g = threadIdx.x; g < c.GG; g += BT) {
        Real a[4];
        const size_t row = (size_t)rir * c.GGp + g;
        ld4(c.lam + row * 4, a);
        double t = (double)a[0] + (double)a[1] + (double)a[2] + (double)a[3];
        out[g] = d_log(t) + (double)c.scl[row] * 0.6931471805599453;
    }
}

// FMA throughput probe: independent FMA chains per thread.
template <typename T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x * (T)1e-7, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3, x4 = x0 + (T)4, x5 = x0 + (T)5,
      x6 = x0 + (T)6, x7 = x0 + (T)7;
    for (int i = 0; i < iters; i++) {
        x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
        x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
    T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == (T)-12345.0) out[blockIdx.x] = s;
}

// ---------------------------------------------------------------------------
// Host-callable launchers (C++ linkage, used by pacc_host.cpp)
// ---------------------------------------------------------------------------
// The model is copied on the stream the kernels run on, so that a launch
// that follows on that stream sees it.
cudaError_t set_model(const DevModel& m, cudaStream_t st) {
    return cudaMemcpyToSymbolAsync(dM, &m, sizeof(DevModel), 0, cudaMemcpyHostToDevice, st);
}

size_t smem_bytes(int N, int BT, int prec, int D) {
    return prec == 0 ? SmemLayout<double>::make(N, BT, D).total : SmemLayout<float>::make(N, BT, D).total;
}

size_t ws_bytes(int n_int, int GGp, int T, int mcmc, int N, int prec) {
    return WsLayout::make(n_int, GGp, T, mcmc, N, prec == 0 ? 8 : 4).total;
}

size_t topo_bytes(int N) { return (size_t)((TopoLayout::make(N).total * 2 + 15) & ~15) + (size_t)N * 8; }

// Kernel instances: FP64 partials one register budget, FP32 partials three
// (variant 0: 128 registers, 1: 168, 2: 255).
int chain_variants(int prec) { return prec == 0 ? 1 : 3; }
int chain_variant_max_threads(int prec, int v) { return (prec == 0 || v == 2) ? 256 : 128; }

template <typename K>
static int occupancy_of(K k, int BT, size_t smem) {
    int nb = 0;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, BT, smem);
    return e == cudaSuccess ? nb : 0;
}

// Resident CTAs per SM of a chain kernel instance for this block size and shared memory.
int chain_occupancy(int prec, int variant, int BT, size_t smem) {
    if (BT > chain_variant_max_threads(prec, variant)) return 0;
    if (prec == 0) return occupancy_of(chain_kernel<double, 256, 1>, BT, smem);
    if (variant == 0) return occupancy_of(chain_kernel<float, 128, 4>, BT, smem);
    if (variant == 1) return occupancy_of(chain_kernel<float, 128, 3>, BT, smem);
    return occupancy_of(chain_kernel<float, 256, 1>, BT, smem);
}

template <typename K>
static cudaError_t launch_of(K k, const ChainParams& p, int grid, int BT, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, BT, smem, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_chain(const ChainParams& p, int grid, int BT, size_t smem, int prec, int variant, cudaStream_t st) {
    if (BT > chain_variant_max_threads(prec, variant)) return cudaErrorInvalidConfiguration;
    if (prec == 0) return launch_of(chain_kernel<double, 256, 1>, p, grid, BT, smem, st);
    if (variant == 0) return launch_of(chain_kernel<float, 128, 4>, p, grid, BT, smem, st);
    if (variant == 1) return launch_of(chain_kernel<float, 128, 3>, p, grid, BT, smem, st);
    return launch_of(chain_kernel<float, 256, 1>, p, grid, BT, smem, st);
}

cudaError_t launch_loglik(const ChainParams& p, const int32_t* z, double c_rate, double n_rate, double* out, int BT,
                          size_t smem, int prec, cudaStream_t st) {
    if (prec == 0) {
        cudaFuncSetAttribute(loglik_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        loglik_kernel<double><<<1, BT, smem, st>>>(p, z, c_rate, n_rate, out);
    } else {
        cudaFuncSetAttribute(loglik_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        loglik_kernel<float><<<1, BT, smem, st>>>(p, z, c_rate, n_rate, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_pmatrix(int n, const double* d, const double* r, double* out, cudaStream_t st) {
    pmatrix_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, d, r, out);
    return cudaGetLastError();
}

cudaError_t launch_stream(uint32_t seed, uint64_t w0, int n, uint32_t* out, cudaStream_t st) {
    stream_kernel<<<(n + 255) / 256, 256, 0, st>>>(seed, w0, n, out);
    return cudaGetLastError();
}

cudaError_t launch_fma_probe(int prec, int grid, int BT, int iters, void* out, cudaStream_t st) {
    if (prec == 0) fma_probe_kernel<double><<<grid, BT, 0, st>>>((double*)out, iters, 0.9999999, 1e-7);
    else fma_probe_kernel<float><<<grid, BT, 0, st>>>((float*)out, iters, 0.9999f, 1e-4f);
    return cudaGetLastError();
}

}  // namespace pacc
