/*
 * pacc.h — C ABI of phyloacc-gb300: PhyloAcc-ST's per-element Bayesian MCMC
 * (three models per element, marginal likelihoods and posteriors of the
 * latent conservation states) on one NVIDIA GB300 GPU.
 *
 * The ABI replaces the per-element seam of PhyloAcc-ST
 *   BPP_C(c, prof, bpp, gapchar, missing_thres, filter&, verbose, consToMis,
 *         prune, revgap, min_length)                (src/PhyloAcc-ST/bpp_c.hpp:143)
 *   -> initMCMC -> Gibbs -> Eval2 -> Output_init    (src/PhyloAcc-ST/main.cpp:459-494)
 * driven by the OpenMP loop over element ids       (src/PhyloAcc-ST/main.cpp:452)
 * and the shared read-only model object BPP         (src/PhyloAcc-ST/bpp.hpp:173-404).
 *
 * Conventions
 *   - Plain C types, caller-owned buffers, no exceptions, no exit().
 *   - Node numbering is PhyloAcc's: leaves 0..S-1 and internal nodes S..N-1
 *     in postorder of the Newick tree, root N-1, N = 2S-1
 *     (src/PhyloAcc-ST/newick.cpp:382-400).  children[2*i+k] lists the
 *     children of node i in increasing id order (src/PhyloAcc-ST/bpp.cpp:105-117),
 *     -1 for leaves.
 *   - Model index m in results: 0 = M0 (null, resZ 0), 1 = M1 (acceleration
 *     off the conserved lineages, resZ 2), 2 = M2 (full, resZ 1)
 *     (src/PhyloAcc-ST/main.cpp:362-364, bpp.cpp:581,590-598).
 *   - Every function returning int returns a pacc_status code.
 *   - A context is driven by one host thread at a time; distinct contexts are
 *     independent and may be used from different threads.
 */
#ifndef PACC_H
#define PACC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PACC_ABI_VERSION 1
#define PACC_MAX_SPECIES 512

typedef enum pacc_status {
    PACC_OK = 0,
    PACC_FILTERED = 1,          /* element dropped by MIN_LEN / CONSERVE_PROP / trimming (bpp_c.hpp:158-162,288-292,369-373) */
    PACC_NAN_LIKELIHOOD = 2,    /* a marginal likelihood was NaN ("failure", bpp_c2.cpp:339-348) */
    PACC_SAMPLER_ERROR = 3,     /* no category could be drawn ("Sample Tg error", bpp_c.cpp:686-696,727-730) */
    PACC_OOM = 4,               /* device or host allocation failed / budget too small */
    PACC_TIMEOUT = 5,           /* a bounded device wait expired */
    PACC_EINVAL = 6,            /* invalid argument */
    PACC_ECUDA = 7,             /* CUDA runtime error */
    PACC_EBUSY = 8,             /* nothing to poll yet / queue full */
    PACC_EUNSUPPORTED = 9       /* option outside the supported model (e.g. INDEL > 0) */
} pacc_status;

typedef enum pacc_precision {
    PACC_FP64 = 0,              /* plain path: one CTA per element chain, FP64 partials, partial re-pruning */
    PACC_FP32 = 1,              /* the same layout with FP32 partials (power-of-two rescaling, integer
                                   exponents), FP64 log-likelihood sums and chain arithmetic */
    PACC_FP64_BATCHED = 2,      /* warp-per-chain layout with FP64 partials (checks it draw for draw) */
    PACC_FP32_WARP = 3          /* warp-per-chain layout with FP32 partials */
} pacc_precision;

/* Tree, rate matrix and species sets: the content of the .mod file plus the
 * OUTGROUP / CONSERVE keys (bpp.hpp:173-404). */
typedef struct pacc_model {
    int32_t n_species;            /* S */
    const int32_t* children;      /* [2*N] */
    const double* distances;      /* [N] branch length above node i (parsed as float, newick.cpp:185,300,325) */
    const double* pi;             /* [4] BACKGROUND */
    const double* rate_matrix;    /* [16] RATE_MAT, row-major */
    const int32_t* outgroup;      /* species ids; a name not found in the tree maps to S (bpp.hpp:303-308) */
    int32_t n_outgroup;
    const int32_t* conserve;      /* species ids (bpp.hpp:237-242) */
    int32_t n_conserve;
} pacc_model;

/* Run options.  pacc_default_opts() gives PhyloAcc-ST's defaults
 * (src/PhyloAcc-ST/main.cpp:36-90). */
typedef struct pacc_opts {
    int32_t burnin;               /* BURNIN   (200) */
    int32_t mcmc;                 /* MCMC     (800) */
    int32_t adapt_freq;           /* ADAPT_FREQ (500) */
    uint32_t seed;                /* SEED (5): every element's stream starts from it */
    double init_conserve_rate;    /* INIT_CONSERVE_RATE (0.5) */
    double init_acce_rate;        /* INIT_ACCE_RATE (1) */
    double conserve_prior_a;      /* CONSERVE_PRIOR_A (5) */
    double conserve_prior_b;      /* CONSERVE_PRIOR_B (0.04) */
    double acce_prior_a;          /* ACCE_PRIOR_A (10) */
    double acce_prior_b;          /* ACCE_PRIOR_B (0.2) */
    int32_t ropt;                 /* ROPT (1) */
    double cub;                   /* CUB (1) */
    double nlb;                   /* NLB (0.6) */
    double init_lrate;            /* INIT_LRATE (0.3) */
    double init_lrate2;           /* INIT_LRATE2 (0.1); forced to 0 when HYPER_LRATE2_A == 0 (main.cpp:286) */
    double init_grate;            /* INIT_GRATE (0.5) */
    double hyper_lrate_a, hyper_lrate_b;     /* (1, 9) */
    double hyper_grate_a, hyper_grate_b;     /* (3, 1) */
    double hyper_lrate2_a, hyper_lrate2_b;   /* (1, 9); a == 0 selects the Dollo model */
    double conserve_prop;         /* CONSERVE_PROP (0.8) */
    double gap_prop;              /* GAP_PROP (0.8) */
    double cons_to_mis;           /* CONSTOMIS (0.01) */
    int32_t gapchar;              /* GAPCHAR ('-') */
    int32_t prune_tree;           /* PRUNE_TREE (0) */
    double trim_gap_percent;      /* TRIM_GAP_PERCENT (1 = off) */
    int32_t min_len;              /* MIN_LEN (50) */
    double indel;                 /* INDEL (0); only 0 is supported */
    /* --- GPU keys (no counterpart in PhyloAcc-ST) --- */
    int32_t precision;            /* pacc_precision (PACC_FP64) */
    int32_t device;               /* CUDA device ordinal (0) */
    int64_t memory_budget_bytes;  /* device bytes the context may hold for chain state (0 = 25% of free);
                                     pacc_gbgc_run: for one launch's traces (0 = 16 GB) */
    int32_t max_resident;         /* max chains resident at once (0 = derived from the budget) */
    int32_t sweeps_per_launch;    /* MCMC iterations per kernel launch (0 = run chains to completion) */
    int32_t trace_iters;          /* record the first trace_iters iterations of every model (0 = off) */
    int32_t block_threads;        /* threads per chain CTA (0 = chosen by the trial-launch tuner:
                                     the fastest of a few threads-per-chain / registers-a-thread /
                                     chains-per-SM shapes on a short trial of the first batch,
                                     remembered per device, taxon count and precision; results do
                                     not depend on the shape) */
    int32_t use_graphs;           /* capture the sweep launches in a CUDA graph (1) */
    int32_t columns_per_lane;     /* batched kernel: alignment columns each lane carries (1, 2 or 4;
                                     0 = autotuned) */
    int32_t chain;                /* CHAIN > 1: index of this chain, 0 = the first.  A later chain
                                     runs every element again from SEED, starting from Z = 0 on
                                     every node (main.cpp:445, bpp_c.cpp:138-151); PACC_FP64 and
                                     PACC_FP32 only */
    int32_t sample_hyper;         /* SAMPLE_HYPER chain (main.cpp:466-494): only the full model M2
                                     runs, from the batch's start states, and every result returns
                                     its end state; PACC_FP64 and PACC_FP32 without serving */
    int64_t serve_idle_ns;        /* serving on the CTA layout: a block of the persistent launch that
                                     has waited this long for work returns (0 = 30 s); elements
                                     published after every block left are taken by the next launch */
    int32_t register_budget;      /* CTA kernel with FP32 partials: registers a thread, 128 (four
                                     128-thread chains per SM), 168 (three) or 255 (two); 0 = chosen
                                     together with block_threads by a trial-launch tuner */
    int32_t reserved0;
} pacc_opts;

/* A batch of elements.  Element e's alignment block is n_species rows of
 * lengths[e] bytes, rows in tree leaf order (the order MatchProfAndTree
 * produces, bpp.cpp:133-184), lower-case as LoadPhyloProfiles stores it
 * (profile.cpp:48,60).  The bytes are copied before pacc_submit returns. */
typedef struct pacc_element_batch {
    int32_t n_elements;
    const int64_t* element_no;    /* [n] value written in the "No." column */
    const int32_t* lengths;       /* [n] alignment columns of each element */
    const int64_t* offsets;       /* [n] byte offset of each block in `bases` */
    const uint8_t* bases;
    /* SAMPLE_HYPER chains (opts.sample_hyper): each element's start state, the
       bpp.cur_Z[1] / cur_*rate of bpp_c.cpp:148-177, or NULL for the first
       chain's start (Z = 1 on the tree's nodes; the INIT_* rates) */
    const int8_t* start_z;        /* [n*N] */
    const double* start_rates;    /* [n*5]: n, c, g, l, l2 */
} pacc_element_batch;

/* Per-model summary (one row of _rate_postZ_M*.txt plus _elem_lik.txt fields). */
typedef struct pacc_model_result {
    double loglik;                /* marginal log-likelihood from Eval2 (bpp_c2.cpp:14-353) */
    double max_loglik;            /* max of the traced full log-likelihood after burn-in (bpp_c.cpp:809-814) */
    double n_rate, c_rate, g_rate, l_rate, l2_rate;  /* posterior medians (bpp_c2.cpp:742-755) */
    int32_t failure;              /* NaN marginal likelihood */
    int32_t n_configs;            /* Z configurations found by Eval2 */
} pacc_model_result;

/* Optional per-iteration trace (first trace_iters iterations of each model). */
typedef struct pacc_trace {
    double* loglik;               /* [3][T]  trace_loglik */
    double* n_rate;               /* [3][T] */
    double* c_rate;               /* [3][T] */
    double* g_rate;               /* [3][T] */
    double* l_rate;               /* [3][T] */
    double* l2_rate;              /* [3][T] */
    int8_t* z;                    /* [3][T][N] */
} pacc_trace;

typedef struct pacc_result {
    int64_t element_no;
    int32_t status;               /* PACC_OK, PACC_FILTERED, PACC_NAN_LIKELIHOOD, PACC_SAMPLER_ERROR */
    int32_t n_nodes;              /* N */
    pacc_model_result model[3];   /* M0, M1, M2 */
    int32_t* max_z;               /* caller buffer [3*N] or NULL: Max_Z per model (bpp.cpp:607-614) */
    double* post_z;               /* caller buffer [3*N*4] or NULL: countZ/MCMC per model (bpp_c2.cpp:757-781) */
    pacc_trace trace;             /* caller buffers or NULL pointers */
    double latency_ms;            /* submit -> result available (serving) */
    double device_ms;             /* time the element's chain spent on the device */
    /* SAMPLE_HYPER chains: the state where M2's chain stopped (bpp_c.cpp:475-485) */
    int8_t* end_z;                /* caller buffer [N] or NULL */
    double end_rates[5];          /* n, c, g, l, l2 */
} pacc_result;

typedef struct pacc_ctx pacc_ctx;

/* Defaults of PhyloAcc-ST's driver plus the GPU keys. */
void pacc_default_opts(pacc_opts* opts);

/* Build a context: validates the tree, decomposes RATE_MAT in FP64
 * (replaces eig_gen/inv at bpp.hpp:357-362), builds the null-rate
 * transition cache (bpp.hpp:366-397) and the upper/upper_conserve sets
 * (bpp.hpp:303-310), and reserves device memory against the budget. */
pacc_ctx* pacc_create(const pacc_model* model, const pacc_opts* opts, int* status);

/* Queue a batch (replaces the element loop of main.cpp:452-500).  Columns
 * are encoded, trimmed and the tree pruned per element on the host
 * (bpp_c.hpp:204-428); elements are admitted to the device as chain slots
 * and memory free up.  Serving on the CTA layout sizes its slots for at
 * least 5,120 columns at the first submit; a later element longer than that
 * first lets the running chains finish, then the slots are made again for
 * it.  Returns PACC_OK or an error; per-element outcomes are reported by
 * pacc_poll. */
int pacc_submit(pacc_ctx* ctx, const pacc_element_batch* batch);

/* Advance the device and collect up to max finished elements into out.
 * Returns the number written (>= 0) or a negative pacc_status. */
int pacc_poll(pacc_ctx* ctx, pacc_result* out, int max);

/* Block until every submitted element has finished. */
int pacc_sync(pacc_ctx* ctx);

/* Number of submitted elements whose results have not been polled yet. */
int pacc_pending(pacc_ctx* ctx);

/* Convenience: submit + sync + poll for one batch; out[i] matches batch order. */
int pacc_run(pacc_ctx* ctx, const pacc_element_batch* batch, pacc_result* out);

void pacc_destroy(pacc_ctx* ctx);

/* Last error text of the context (or of the last failed pacc_create when ctx is NULL). */
const char* pacc_last_error(pacc_ctx* ctx);

/* Device counters of the last pacc_sync/pacc_run: work units actually performed. */
typedef struct pacc_counters {
    double edge_updates_internal;  /* parent *= P * child-partial (internal child): 36 flop each */
    double edge_updates_leaf;      /* parent *= column of P (leaf child): 4 (8 ambiguous) flop each */
    double column_loglik;          /* per-column root sums + logs */
    double tg_draws;               /* internal-base categorical draws */
    double z_draws;                /* latent-state draws */
    double pmatrix_builds;         /* branch transition matrices built on device */
    double iterations;             /* MCMC iterations run (all models) */
    double kernel_ms;              /* summed duration of the chain kernels (CUDA events) */
    double flop;                   /* algorithmic FP work of the prunes, counted from the above */
    double phase_cycles[8];        /* SM cycles summed over chains.  CTA kernel: monitor, internal-base
                                      pass (with the emission histogram), emission sums, Z filter,
                                      Z-change likelihood, accelerated-rate MH, conserved-rate MH,
                                      transitions.  Warp kernel: internal-base pass, emission sums, Z
                                      filter, Z-change likelihood, accelerated-rate MH, conserved-rate
                                      MH, monitor/transitions, model init + Eval2 + output.
                                      gBGC chain (pacc_gbgc_run): monitor + model set-up, expected
                                      counts, initial_prob_back, branch matrices of the rate
                                      proposals, the rest of sample_rates, Update_ZB, pruning,
                                      ELBO + update_rates' MH */
    double serve_idle_exits;       /* serving (CTA layout): blocks that left a launch on the idle bound */
} pacc_counters;
int pacc_get_counters(pacc_ctx* ctx, pacc_counters* out);

/* Launch shape of the CTA-per-chain kernel (no counterpart in the reference):
 * threads per chain, registers a thread, resident chains per SM and the
 * duration of the tuner's trial launches (0 when the shape was fixed by the
 * options or taken from an earlier context).  Zeros before the first launch
 * or on the warp-per-chain layouts. */
int pacc_get_launch_shape(pacc_ctx* ctx, int32_t* block_threads, int32_t* registers, int32_t* chains_per_sm,
                          double* trial_ms);

/* --- The gBGC model (PhyloAcc-ST-GBGC, src/PhyloAcc-ST-GBGC/SRC) --- */

/* Options of the gBGC model's chains.  pacc_gbgc_default_opts() gives that
 * program's defaults (main.cpp:36-81; bpp.cpp:217-219; bpp_c.hpp:365-370). */
typedef struct pacc_gbgc_opts {
    int32_t burnin;               /* BURNIN (200) */
    int32_t mcmc;                 /* MCMC (800) */
    uint32_t seed;                /* SEED (7728): every element's stream starts from it */
    int32_t gapchar;              /* GAPCHAR ('*'): the character counted as missing */
    double conserve_rate;         /* CONSERVE_RATE (-2): initial conserved selection */
    double acce_rate;             /* ACCE_RATE (0): initial accelerated selection */
    double init_gc;               /* initial GC bias (3; cur_nGB, bpp.cpp:219) */
    double conserve_prior_a;      /* CONSERVE_PRIOR_A (5): -selection_c ~ Gamma(a, b) */
    double conserve_prior_b;      /* CONSERVE_PRIOR_B (0.4) */
    double acce_prior_a;          /* ACCE_PRIOR_A (5): selection_n + shift ~ Gamma(a, b) */
    double acce_prior_b;          /* ACCE_PRIOR_B (0.4) */
    double acce_prior_shift;      /* nprior_c (2, bpp.hpp:199) */
    double gc_prior_a;            /* nGBprior_a (4): GC bias ~ Gamma(a, b) */
    double gc_prior_b;            /* nGBprior_b (0.8) */
    double gc_prior_c;            /* nGBprior_c (0.2): prior probability of B = 1 on a branch */
    double prep_lrate;            /* PREP_LRATE (0.1): P(Z 1 -> 2) */
    double prep_grate;            /* PREP_GRATE (0.8): P(Z 0 -> 1) */
    double cons_to_mis;           /* CONSTOMIS (0.01) */
    double ncons_to_mis;          /* nconsToMis (0.1) */
    double missing_thres;         /* GAP_PROP (0.8): a taxon with more gap characters is missing */
    double conserve_prop;         /* CONSERVE_PROP (0.8) */
    double prop_c, prop_n, prop_gc;   /* proposal widths (1.2, 1.2, 0.2; bpp_c.hpp:365-370) */
    const int32_t* target;        /* TARGETSPECIES node ids (M2 lets only these leaves accelerate) */
    int32_t n_target;
    int32_t chain;                /* chain k of the CHAIN loop (main.cpp:372): a later chain starts
                                     every node, inside the element's tree or not, from Z = 0
                                     (bpp.cur_Z, never written without SAMPLE_HYPER; bpp_c.cpp:128-131) */
} pacc_gbgc_opts;

void pacc_gbgc_default_opts(pacc_gbgc_opts* opts);

/* One element's gBGC results: the three models run M0 (null), M2 (res),
 * M1 (full) from one stream, as main.cpp:383-412 does; arrays are indexed by
 * model 0 = M0, 1 = M1, 2 = M2. */
typedef struct pacc_gbgc_result {
    int64_t element_no;
    int32_t status;               /* PACC_OK or PACC_FILTERED */
    int32_t root;                 /* the element's root after the outgroup-path collapse */
    double loglik_null;           /* Eval2 of M0 (bpp_c2.cpp:29-286): loglik_NUll */
    double loglik_res;            /* Eval2 of M2: loglik_RES */
    double loglik_all;            /* Eval2 of M1: loglik_all */
    double max_loglik[3];         /* loglik_Max1..3: the best full log-likelihood after burn-in */
    double rates[3][3];           /* posterior medians: [model][n_rate, c_rate, gBC] (bpp_c2.cpp:603-615) */
    double device_ms;
    /* caller-provided outputs (NULL to skip) */
    int32_t* max_z;               /* [3][N] Max_Z */
    int8_t* max_b;                /* [3][N] Max_B */
    double* post_b;               /* [3][N] fraction of samples with B = 1 */
    double* post_z;               /* [3][N][4] fractions of Z = -1, 0, 1, 2 (missing branches: 1 in column 0) */
    double* trace;                /* [3][burnin+mcmc][4 + 2N]: full loglik, n, c, gBC, B[N], Z[N] */
} pacc_gbgc_result;

/* Run every element of the batch through the gBGC model's three chains on
 * the device (one CTA an element; the element loop of main.cpp:383-412 with
 * BPP_C, initMCMC, Gibbs, Eval2 and Output_init per model).  The context gives
 * the tree, rate matrix, outgroup and conserved sets and the precision of the
 * partials (PACC_FP32 / PACC_FP32_WARP: FP32, else FP64), the device memory
 * for one launch's traces (memory_budget_bytes, 0 = 16 GB; more elements run
 * as several launches) and the chain kernel's register budget
 * (register_budget 168: three CTAs an SM, else 96 registers and five); its
 * other options are not used.  Eval2 and Output_init run on the host from
 * the device's traces.  Returns when every element's result is written. */
int pacc_gbgc_run(pacc_ctx* ctx, const pacc_gbgc_opts* opts, const pacc_element_batch* batch,
                  pacc_gbgc_result* out);

/* Serving form of pacc_gbgc_run: elements are admitted while others run.  A
 * persistent chain kernel (one CTA an element) takes elements from a queue
 * the host appends to; submit preprocesses the batch and queues it (a change
 * of options, precision or a longer element than the serving slots hold
 * first lets the running elements finish and re-creates the slots); poll
 * collects finished elements (Eval2 and the tables on the host) and writes
 * up to max results, in completion order, into out, copying the per-node
 * arrays into the buffers out[i].max_z / max_b / post_b / post_z point to
 * (when non-null; traces are not kept); out[i].device_ms is the element's
 * time from submit to collection.  sync returns when every submitted element
 * has finished (their results stay for poll).  The blocks leave after
 * opts.serve_idle_ns of the context without work; opts.max_resident (> 0)
 * caps the device slots (default: two per resident CTA), within
 * opts.memory_budget_bytes (0 = a quarter of the free device memory). */
int pacc_gbgc_submit(pacc_ctx* ctx, const pacc_gbgc_opts* opts, const pacc_element_batch* batch);
int pacc_gbgc_poll(pacc_ctx* ctx, pacc_gbgc_result* out, int max);
int pacc_gbgc_sync(pacc_ctx* ctx);

/* --- Kernel-level entry points used by parity tests (same kernels as the chain) --- */

/* (a) P^T = eigeninv * diag(exp(lambda*d*r)) * eigenvec for n branch lengths
 * d[i] and rates r[i], FP64 on the device.  out: [n][16] row-major (child, parent). */
int pacc_debug_pmatrix(pacc_ctx* ctx, int n, const double* d, const double* r, double* out);

/* The same P^T matrices as pacc_debug_pmatrix, computed without allocating.
 * This entry point has no counterpart in the reference (PhyloAcc-ST builds
 * its matrices on the host with Armadillo); it exists for callers that must
 * not allocate device memory at that moment: a process whose device memory
 * is fully committed (a serving context holding its whole budget in chain
 * slots), or one that cannot afford the device-wide synchronisation that
 * cudaFree implies while other streams are busy.
 * Working memory is a fixed file-scope device array of PACC_NOALLOC_MAX_PAIRS
 * (distance, rate) pairs and their matrices (about 590 KB per device); larger
 * requests return PACC_EINVAL.  Nothing in the scratch has to start at zero:
 * the kernel writes every matrix that is copied back.
 * Set-up: every call looks the scratch's device address up with
 * cudaGetSymbolAddress; the first call on a device also loads the module
 * there.  Make the first call from ordinary code, before any stream capture.
 * The call runs on the context's own second stream, so a serving launch of
 * the same context does not hold it back (the serving launch leaves one
 * chain slot of the GPU free for it); a context whose model is not the
 * device's current one first waits for the other context's launch.
 * The scratch is shared by every context on a device: calls that overlap on
 * one device (two threads, or two contexts' streams) race on it.
 * n: 1..PACC_NOALLOC_MAX_PAIRS; d, r, out: host arrays as for pacc_debug_pmatrix.
 * Returns when out is written. */
#define PACC_NOALLOC_MAX_PAIRS 4096
int pacc_pmatrix_noalloc(pacc_ctx* ctx, int n, const double* d, const double* r, double* out);

/* The likelihood engine of the PhyloAcc-ST-GBGC model (selection plus
 * GC-biased gene conversion) on one element at one state, on the device.
 * It replaces, for that model (src/PhyloAcc-ST-GBGC/SRC):
 *   - the BPP_C constructor's column encoding, missing taxa, conserved-species
 *     filter and outgroup-path collapse (bpp_c.hpp:153-379, bpp_c.cpp:53-111);
 *   - getRate (bpp_c.cpp:13-30) and init_cache_TM (bpp_c.cpp:1563-1621): the six
 *     classes of branch matrices, null, conserved, accelerated, each without
 *     and with the GC bias, built here by Pade scaling and squaring in FP64;
 *   - Update_Tg's pruning pass and per-column log-likelihood (bpp_c.cpp:477-540)
 *     and its expected (child base, parent base) counts (bpp_c.cpp:541-596).
 * bases: S rows of length lower-case characters in tree leaf order; gapchar
 * and missing_thres as the model's GAPCHAR ('*') and MISSING_THRES (0.8);
 * the conserved-species filter uses the context's conserve_prop.
 * z: [N] 0 null / 1 conserved / 2 accelerated (not 2 on the outgroup path);
 * b: [N] 0 or 1 (the gBGC flag); both read on the element's branches only;
 * sel_c, sel_n: conserved and accelerated selection; gc_bias: the GC bias.
 * Partials are FP32 when the context's precision is PACC_FP32 or
 * PACC_FP32_WARP, else FP64.
 * Out: logp [6][N][16] log P(child | parent) in the class order above (0 on
 * branches not built: missing ones, and the accelerated classes on the
 * outgroup path); col [length] per-column log-likelihoods; counts [N][16]
 * expected counts summed over columns (the root's posterior in entries j*4);
 * root (the element's root after the collapse); missing [N]; filtered.
 * Returns PACC_FILTERED (outputs other than missing and filtered untouched)
 * for a filtered element. */
int pacc_gbgc_engine(pacc_ctx* ctx, const uint8_t* bases, int32_t length, int32_t gapchar, double missing_thres,
                     const int32_t* z, const int32_t* b, double sel_c, double sel_n, double gc_bias, double* logp,
                     double* col, double* counts, int32_t* root, uint8_t* missing, int32_t* filtered);

/* (b) Per-column log-likelihood of one element for a given Z (int32 [N]) and
 * conserved/accelerated rates, using the chosen precision's pruning kernel.
 * out: [columns after trimming]; returns the column count via *n_cols. */
int pacc_debug_loglik(pacc_ctx* ctx, const uint8_t* bases, int32_t length, const int32_t* z,
                      double c_rate, double n_rate, double* out, int32_t* n_cols);

/* Per-element column encoding (bpp_c.hpp:204-264): Tg codes after trimming,
 * [n_cols][N] int8 (-1 ambiguous, 0..3 base, 4 gap, 5 other; internal nodes
 * set to 4 where both children are >= 4), plus the missing flags [N] and the
 * pruned-tree root.  For bit-exact checks of the host preprocessing. */
int pacc_debug_encode(pacc_ctx* ctx, const uint8_t* bases, int32_t length, int8_t* tg_out,
                      int32_t* n_cols, uint8_t* missing_out, int32_t* root_out, int32_t* filtered);

/* Site patterns of one element after trimming: pattern_of[g] (int32 [n_cols])
 * is the pattern of column g, patterns numbered in order of first occurrence;
 * weights[p] (int32, room for n_cols) counts the columns of pattern p.
 * Host only; for bit-exact checks of the compression. */
int pacc_debug_patterns(pacc_ctx* ctx, const uint8_t* bases, int32_t length, int32_t* pattern_of,
                        int32_t* weights, int32_t* n_cols, int32_t* n_patterns);

/* Philox stream words w0 .. w0+n-1 generated on the device. */
int pacc_debug_stream(uint32_t seed, uint64_t w0, int n, uint32_t* out);

/* Measured FMA throughput of this GPU, FLOP/s: fp64 and fp32 (FMA = 2 flop). */
int pacc_measure_fma_peak(int device, double* fp64_flops, double* fp32_flops);

#ifdef __cplusplus
}
#endif
#endif /* PACC_H */
