// pacc_dev.h — data shared between the host preprocessing and the chain kernel.
#pragma once
#include <stdint.h>

#ifndef __CUDACC__
#define __host__
#define __device__
#endif

namespace pacc {

static const int KB = 4;          // bases (num_base with INDEL == 0)
static const int NSYM = 10;       // emission symbols: 0..3 base, 4..9 ambiguity codes r y k m s w
static const int MAX_NODES = 511; // N = 2S-1 with S <= 256

// Leaf column codes (one byte per taxon and column).
enum LeafCode : uint8_t {
    CODE_A = 0, CODE_C = 1, CODE_G = 2, CODE_T = 3,
    CODE_GAP = 4,   // GAPCHAR: Tg = 4 (bpp_c.hpp:259)
    CODE_OTHER = 5, // n and anything else: Tg = 5 (bpp_c.hpp:260)
    CODE_R = 6, CODE_Y = 7, CODE_K = 8, CODE_M = 9, CODE_S = 10, CODE_W = 11  // Tg = -1
};

// Two-hot masks of the ambiguity codes r y k m s w (bpp_c.hpp:230-248):
// r = a|g (0x5), y = c|t (0xA), k = g|t (0xC), m = a|c (0x3), s = c|g (0x6), w = a|t (0x9).
__host__ __device__ inline int ambig_mask(int k) { return (0x963CA5 >> (4 * k)) & 0xF; }

// Model constants (one per context), copied to __constant__ memory.
struct DevModel {
    int S, N;
    double lam[4];
    double evec[16];   // eigenvec = V^T, row-major [i][b]
    double einv[16];   // eigeninv = (V^T)^-1, row-major [a][i]
    double pi[4];
    double log_pi[4];
    // options (main.cpp:36-90)
    int burnin, mcmc, adapt_freq, ropt;
    uint32_t seed;
    double init_c, init_n, cprior_a, cprior_b, nprior_a, nprior_b, cub, nlb;
    double init_l, init_l2, init_g;
    double la, lb, ga, gb, l2a, l2b;
    double cons_to_mis;
    int trace_iters;
    // FP32-partial path: P^T(d r)[a][b] = [a == b] + sum_i A[a][b][i] (exp(lambda_i d r) - 1)
    // with A[a][b][i] = eigeninv[a][i] * eigenvec[i][b] rounded to FP32
    float a32[64];
    // log normalisers lgamma(a) + a log(b) of the conserved and accelerated rate priors
    double kc, kn;
};

// Per-element topology after missing-taxon pruning (bpp_c.hpp:331-428),
// node ids are PhyloAcc's.  Offsets are in int16 units from the start of
// the element's topology block; see host code for the layout.
struct ElemHeader {
    int32_t GG;            // columns after trimming
    int32_t GGp;           // GG rounded up to a multiple of 32
    int32_t root;
    int32_t n_nodes;       // |nodes| (postorder of the pruned tree)
    int32_t n_int;         // |internal_nodes|
    int32_t n_hlev;        // bottom-up levels (by height) of non-leaf nodes
    int32_t n_dlev;        // top-down levels (by depth) below the root
    int32_t tg_draws;      // stream words used by one internal-base pass (prefix[GG])
    int64_t codes_off;     // byte offset of codes [S][GGp]
    int64_t codes_t_off;   // byte offset of codes by column [GGp][SP] (SP = S rounded up to 16)
    int64_t tg_off;        // byte offset of initial internal Tg [n_int][GGp] (int8)
    int64_t prefix_off;    // byte offset of draw prefix [GG+1] (int32)
    int64_t topo_off;      // byte offset of the int16 topology block
    int64_t element_no;
    int32_t filtered;
    int32_t SP;            // taxa per column row in codes_t (multiple of 16)
    int32_t stack_depth;   // partials pending at once in the stack-order traversal
    int32_t GGu;           // distinct site patterns among the GG columns
    int64_t pcodes_off;    // byte offset of the patterns by column [GGu rounded up to 32][SP]
    int64_t pw_off;        // byte offset of the pattern weights [GGu] (int32)
    int64_t pof_off;       // byte offset of the pattern of each column [GG] (int32)
};

// Layout of the int16 topology block (each array length N unless noted).
struct TopoLayout {
    int nodes, internal, c2a, c2b, par, irank, pos, missing, upc, upcc, hlev_start, hlev_nodes, dlev_start,
        dlev_nodes, sord, sflag, total;
    __host__ __device__ static TopoLayout make(int N) {
        TopoLayout t;
        int o = 0;
        t.nodes = o; o += N;
        t.internal = o; o += N;
        t.c2a = o; o += N;
        t.c2b = o; o += N;
        t.par = o; o += N;
        t.irank = o; o += N;
        t.pos = o; o += N;
        t.missing = o; o += N;
        t.upc = o; o += N;
        t.upcc = o; o += N;
        t.hlev_start = o; o += N + 1;
        t.hlev_nodes = o; o += N;
        t.dlev_start = o; o += N + 1;
        t.dlev_nodes = o; o += N;
        t.sord = o; o += N;    // internal nodes in a postorder that visits the child needing more stack first
        t.sflag = o; o += N;   // bit 0: the first child's (c2a) partial is on top of the stack at its parent
        t.total = o;
        return t;
    }
};

// Per-model result written by the kernel.
struct DevModelResult {
    double loglik, max_loglik, rates[5];
    int32_t failure, n_configs;
};

struct DevResult {
    DevModelResult model[3];
    int32_t status;
    int32_t pad;
    double device_ms;
};

// Work counters accumulated by the kernel (atomicAdd per CTA per element).
struct DevCounters {
    unsigned long long edge_internal, edge_leaf, col_ll, tg_draws, z_draws, pmat, iters;
    unsigned long long phase_cycles[8];  // cycles per phase (summed over chains)
    unsigned long long idle_exits;       // serving: blocks that left on the idle bound
};

// One internal node of the pruned tree, in postorder, as the batched kernel
// reads it (one 16-byte shared-memory load per node and column).
struct NodeRec {
    int16_t c0, c1;      // child node ids
    int16_t r0, r1;      // internal rank of a child (-1 for a leaf)
    int8_t m0, m1;       // child missing (skipped by the prune)
    int8_t missing;      // this node missing
    int8_t is_root;
    int16_t self;        // node id
    int16_t prank;       // internal rank of the parent (-1 for the root)
};

// Parameters of one chain-kernel launch.
struct ChainParams {
    const ElemHeader* hdr;     // [n_elem]
    const uint8_t* blob;       // element data (codes, initial Tg, draw prefix, topology)
    int n_elem;
    int* next_elem;            // work counter (atomic)
    const int32_t* order;      // element claimed by work item i (longest first), or null
    DevResult* results;        // [n_elem]
    int32_t* max_z;            // [n_elem][3][N]
    double* post_z;            // [n_elem][3][N][4]
    double* tr_d;              // [n_elem][3][6][TI] (loglik, n, c, g, l, l2) or null
    int8_t* tr_z;              // [n_elem][3][TI][N] or null
    char* ws;                  // per-CTA workspace
    size_t ws_stride;
    int n_int_max, GGp_max;
    int stack_cap;             // rows of the prune's shared-memory stack (>= every element's stack_depth)
    int trial_burn, trial_mcmc;  // > 0: a tuning trial with these chain lengths instead of the model's
    DevCounters* counters;
    // stream mode (serving): CTAs take slots from a queue the host appends to
    // while the kernel runs; element data and results are indexed by slot.
    int stream;                      // 0: the n_elem elements of this launch; 1: the queue
    int* q_head;                     // device: next queue position to take (atomic)
    const volatile int* q_tail;      // host-mapped: queue positions published so far
    const volatile int* q_slot;      // host-mapped: slot of queue position i (ring of q_cap)
    int q_cap;
    volatile int* done_flag;         // host-mapped, per slot: set to 1 once the slot's results are written
    const volatile int* q_stop;      // host-mapped: nonzero asks the blocks to return when idle
    long long idle_ns;               // safety bound: a block idle this long returns even without q_stop
    int z_start_zero;                // a later chain of a CHAIN > 1 run: Z starts at 0 on every node
    // SAMPLE_HYPER chains: models from first_model (2: M2 only); per element
    // the start state (start_z[e*N] == -128: the first chain's Z) and the
    // state where M2's chain stopped
    int first_model;
    const int8_t* start_z;           // [n][N]
    const double* start_rates;       // [n][5] n, c, g, l, l2
    int8_t* end_z;                   // [n][N]
    double* end_rates;               // [n][5]
};

// ---- batched (warp-per-chain) kernel ----
enum { PH_INIT = 0, PH_RUN = 1, PH_DONE = 2, PH_EMPTY = 3 };

struct SlotState {
    int32_t elem, phase, mi, m;
    int32_t resZ, pad0;
    uint64_t pos;
    double rate_n, rate_c, gr, lr, lr2;
    double prop_n, prop_c;
    int32_t acc_n, acc_c;
    double loglik, maxll;
    int32_t max_m, status;
    int64_t start_clock;
    int64_t iters;
};

struct BatchParams {
    const ElemHeader* hdr;
    const uint8_t* blob;
    SlotState* slots;
    int n_slots;
    char* slot_ws;            // per-slot: Z, maxz, class tables, traces
    size_t slot_ws_stride;
    char* grp_ws;             // per-warp scratch for Eval2
    size_t grp_ws_stride;
    int sweeps;               // iterations per slot per launch (<= 0: until done)
    DevResult* results;       // by element index
    int32_t* max_z;
    double* post_z;
    double* tr_d;
    int8_t* tr_z;
    DevCounters* counters;
    int* n_done;              // number of slots that reached PH_DONE in this launch
    int* next_slot;           // slot queue (atomic)
    int* done_list;           // slots that reached PH_DONE in this launch (n_done entries), or null
    int n_int_max, S_max;
    int stack_depth;          // max over admitted elements
    int GGuP_max;             // pattern capacity of the per-warp partial buffers (multiple of 32)
};


// Parameters of one launch of the gBGC likelihood engine (one element at one
// state of the PhyloAcc-ST-GBGC model).
struct GbgcParams {
    int S, N, GG, GGp, root, n_nodes;   // GGp: columns rounded up to 32 (padding columns allow every base)
    int warps;                          // warps of the engine's CTA
    const int16_t* nodes;               // [n_nodes] postorder of the element's tree (collapsed outgroup path)
    const int16_t* c0;                  // [N] children in that tree (-1: leaf)
    const int16_t* c1;
    const int16_t* parent;              // [N]
    const uint8_t* missing;             // [N]
    const uint8_t* fixed;               // [N] no accelerated class on this branch (the outgroup path)
    const double* dist;                 // [N] branch lengths after the collapse
    const int32_t* cls;                 // [N] matrix class of the branch above the node: Z + 3 B
    const uint8_t* masks;               // [S][GGp] allowed bases of a leaf at a column (bit i: base i)
    double Q0[16], pi[4];
    double sc, sn, gb;                  // conserved / accelerated selection, GC bias
    double* logp;                       // [6][N][16] log P, (child, parent) row-major
    void* pmat;                         // [6][N][16] P in the partials' type
    double* col;                        // [GG] per-column log-likelihood
    double* counts;                     // [N][16] expected (child, parent) base counts
    double* wcounts;                    // [warps][N][16] per-warp sums
    void* part;                         // [N][GGp][4] partials, then marginals
    int32_t* scl;                       // [N][GGp] power-of-two exponents of the partials
};

// ---- the gBGC model's chain kernel ----

// One element of the gBGC chain: its tree after the outgroup-path collapse
// and its leaf columns, as byte offsets into the element's blob.
struct GbgcElemHdr {
    int32_t S, N, GG, GGp, root, n_nodes, n_int, n_hlev, n_dlev;
    int32_t o_nodes, o_c0, o_c1, o_par, o_irank, o_pidx, o_flags;   // int16 / uint8 [N]
    int32_t o_dist;                  // double [N]
    int32_t o_hlev, o_hnodes;        // internal nodes by height: starts [n_hlev + 1], nodes
    int32_t o_dlev, o_dnodes;        // non-root nodes by depth: starts [n_dlev + 1], nodes
    int32_t o_masks;                 // uint8 [S][GGp] allowed bases
    int32_t o_blen, n_blen;          // int16: the branches that are not missing, by length
    int64_t blob_off;
};

enum { GBGC_MISSING = 1, GBGC_UPPER = 2, GBGC_TARGET = 4 };

// Per-CTA workspace of the gBGC chain kernel (byte offsets).  Matrix slots:
// 0 the null class; 1 + 5 q + (k - 1) class k = 1..5 of cache set q = 0..2.
struct GbgcWs {
    size_t lP, pm, post, wc, emis, emis_tmp, lpb, eraw, colsum, part, scl, total;
    static __host__ __device__ size_t up(size_t b) { return (b + 255) & ~(size_t)255; }
    static __host__ __device__ GbgcWs make(int N, int n_int, int GGp, int warps, int rb) {
        GbgcWs w;
        size_t o = 0;
        w.lP = o;       o += up((size_t)16 * N * 16 * 8);
        w.pm = o;       o += up((size_t)16 * N * 16 * rb);
        w.post = o;     o += up((size_t)2 * N * 16 * 8);
        w.wc = o;       o += up((size_t)warps * N * 16 * 8);
        w.emis = o;     o += up((size_t)N * 6 * 8);
        w.emis_tmp = o; o += up((size_t)N * 6 * 8);
        w.lpb = o;      o += up((size_t)N * 6 * 8);
        w.eraw = o;     o += up((size_t)N * 8);
        w.colsum = o;   o += up((size_t)warps * 8);
        w.part = o;     o += up((size_t)2 * n_int * GGp * 4 * rb);
        w.scl = o;      o += up((size_t)2 * n_int * GGp * 4);
        w.total = o;
        return w;
    }
};

struct GbgcChainParams {
    const GbgcElemHdr* hdr;
    const uint8_t* blob;
    int n_elem;
    int* next_elem;
    int T, burn, mcmc;
    uint32_t seed;
    int chain;                // > 0: a later chain of a CHAIN > 1 run (Z starts at 0 everywhere)
    double conserve_rate, acce_rate, init_gc;
    double ca, cb, na, nb, nshift, gca, gcb, gcc;   // priors: conserved, accelerated (+ shift), GC bias
    double lrate, grate, c2m, nc2m, prop_c, prop_n, prop_gc;
    double Q0[16], pi[4];
    const uint8_t* target;    // [N_max] TARGETSPECIES flags
    char* ws;
    size_t ws_stride;
    int N_max, n_int_max, GGp_max;
    // outputs
    double* tr_d;             // [n_elem][3][4][T]: full loglik, n, c, gBC
    int8_t* tr_zb;            // [n_elem][3][T][2][N_max]: Z then B
    int8_t* max_zb;           // [n_elem][3][2][N_max]
    double* max_ll;           // [n_elem][3]
    int32_t* status;          // [n_elem]
    // stream mode (serving): elements come from a queue the host appends to
    // while the kernel runs; element data and outputs are indexed by slot
    int stream;
    int* q_head;                     // device: next queue position to take
    const volatile int* q_tail;      // host-mapped: positions published so far
    const volatile int* q_slot;      // host-mapped: slot of position i (ring of q_cap)
    int q_cap;
    volatile int* done_flag;         // host-mapped, per slot: 1 once the slot's outputs are written
    const volatile int* q_stop;      // host-mapped: nonzero asks idle blocks to return
    long long idle_ns;               // a block idle this long returns even without q_stop
    unsigned long long* idle_exits;  // blocks that left on the idle bound
    unsigned long long* phase;       // [8] cycles per phase (summed over elements), or null
    unsigned long long* flop;        // FP64 flops of the Padé solves (algorithmic count), or null
};

}  // namespace pacc
