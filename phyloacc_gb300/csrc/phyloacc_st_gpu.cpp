// phyloacc-st-gpu — drop-in replacement for the PhyloAcc-ST executable.
//
//     phyloacc-st-gpu <config file>
//
// Reads the same key-value configuration (src/PhyloAcc-ST/main.cpp:100-287),
// the same inputs (.mod tree + rate matrix, FASTA alignment, bed segments,
// optional id list) and writes the same tables that phyloacc.py's snakemake
// rule expects and phyloacc_post.py reads (main.cpp:360-402, bpp.cpp:568-619,
// bpp_c2.cpp:706-785):
//   <PREFIX>_elem_lik.txt, <PREFIX>_M{0,1,2}_elem_Z.txt,
//   <PREFIX>_rate_postZ_M{0,1,2}.txt, <PREFIX>_hyper.txt,
//   <PREFIX>_species_names.txt and, with VERBOSE, <PREFIX>_mcmc_trace_M{m}_{No}.txt.
// The MCMC itself runs on the GPU through the C ABI of include/pacc.h.
// Extra keys (ignored by PhyloAcc-ST): GPU_PRECISION fp64|fp32|fp32_warp|fp64_warp, GPU_DEVICE,
// GPU_BLOCK_THREADS, GPU_MEMORY_BUDGET_GB.
#include <dirent.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "pacc.h"
#include "cli_io.h"

// ---------------------------------------------------------------------------
// configuration (main.cpp:36-287)
// ---------------------------------------------------------------------------
struct Config {
    string phytree, align, segment, id_path, output, prefix = "test";
    string outgroup, target, conserve;
    int batch = -1, chain = 0, num_thread = 1;
    bool verbose = false, sample_hyper = false;
    pacc_opts o;
};

static bool to_bool(const string& s) { return s == "true" || s == "1"; }

static Config load_config(const string& path) {
    Config C;
    pacc_default_opts(&C.o);
    std::ifstream in(path.c_str());
    if (!in) die("Cannot open the parameters file: " + path);
    string line;
    int line_num = 1;
    double lrate2_init = C.o.init_lrate2;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        vector<string> w;
        string word;
        while (ls >> word) w.push_back(word);
        if (w.empty() || w[0][0] == '#') continue;
        if (w.size() != 2) {
            std::cerr << "\nLine " << line_num << " in the parameter file is not formatted correctly: " << line << "\n";
            die("Each line should contain a parameter and a value separated by a space and no other whitespace.\n");
        }
        const string& k = w[0];
        const string& v = w[1];
        pacc_opts& o = C.o;
        if (k == "PHYTREE_FILE") C.phytree = v;
        else if (k == "ALIGN_FILE") C.align = v;
        else if (k == "SEG_FILE") C.segment = v;
        else if (k == "ID_FILE") C.id_path = v;
        else if (k == "BATCH") C.batch = std::stoi(v);
        else if (k == "RESULT_FOLDER") C.output = v;
        else if (k == "PREFIX") C.prefix = v;
        else if (k == "SEED") o.seed = (uint32_t)std::stoi(v);
        else if (k == "INIT_CONSERVE_RATE") o.init_conserve_rate = std::stod(v);
        else if (k == "INIT_ACCE_RATE") o.init_acce_rate = std::stod(v);
        else if (k == "CONSERVE_PRIOR_A") o.conserve_prior_a = std::stod(v);
        else if (k == "CONSERVE_PRIOR_B") o.conserve_prior_b = std::stod(v);
        else if (k == "ACCE_PRIOR_A") o.acce_prior_a = std::stod(v);
        else if (k == "ACCE_PRIOR_B") o.acce_prior_b = std::stod(v);
        else if (k == "ROPT") o.ropt = std::stoi(v);
        else if (k == "CUB") o.cub = std::stod(v);
        else if (k == "NLB") o.nlb = std::stod(v);
        else if (k == "BURNIN") o.burnin = std::stoi(v);
        else if (k == "MCMC") o.mcmc = std::stoi(v);
        else if (k == "ADAPT_FREQ") o.adapt_freq = std::stoi(v);
        else if (k == "INIT_LRATE") o.init_lrate = std::stod(v);
        else if (k == "INIT_LRATE2") lrate2_init = std::stod(v);
        else if (k == "INIT_GRATE") o.init_grate = std::stod(v);
        else if (k == "HYPER_LRATE_A") o.hyper_lrate_a = std::stod(v);
        else if (k == "HYPER_LRATE_B") o.hyper_lrate_b = std::stod(v);
        else if (k == "HYPER_GRATE_A") o.hyper_grate_a = std::stod(v);
        else if (k == "HYPER_GRATE_B") o.hyper_grate_b = std::stod(v);
        else if (k == "HYPER_LRATE2_A") o.hyper_lrate2_a = std::stod(v);
        else if (k == "HYPER_LRATE2_B") o.hyper_lrate2_b = std::stod(v);
        else if (k == "CHAIN") C.chain = std::stoi(v);
        else if (k == "OUTGROUP") C.outgroup = v;
        else if (k == "TARGETSPECIES") C.target = v;
        else if (k == "CONSERVE") C.conserve = v;
        else if (k == "CONSERVE_PROP") o.conserve_prop = std::stod(v);
        else if (k == "GAP_PROP") o.gap_prop = std::stod(v);
        else if (k == "CONSTOMIS") o.cons_to_mis = std::stod(v);
        else if (k == "GAPCHAR") o.gapchar = v[0];
        else if (k == "PRUNE_TREE") o.prune_tree = to_bool(v);
        else if (k == "TRIM_GAP_PERCENT") o.trim_gap_percent = std::stod(v);
        else if (k == "MIN_LEN") o.min_len = std::stoi(v);
        else if (k == "INDEL") o.indel = std::stoi(v);
        else if (k == "INDEL2") {}
        else if (k == "SAMPLE_INDEL") {}
        else if (k == "SAMPLE_HYPER") C.sample_hyper = to_bool(v);
        else if (k == "VERBOSE") C.verbose = to_bool(v);
        else if (k == "NUM_THREAD") C.num_thread = std::stoi(v);
        else if (k == "GPU_PRECISION") {
            std::string u = v;
            for (auto& ch : u) ch = (char)std::tolower((unsigned char)ch);
            o.precision = u == "fp32" ? PACC_FP32 : u == "fp32_warp" ? PACC_FP32_WARP
                        : u == "fp64_warp" ? PACC_FP64_BATCHED : PACC_FP64;
        }
        else if (k == "GPU_DEVICE") o.device = std::stoi(v);
        else if (k == "GPU_BLOCK_THREADS") o.block_threads = std::stoi(v);
        else if (k == "GPU_COLUMNS_PER_LANE") o.columns_per_lane = std::stoi(v);
        else if (k == "GPU_MEMORY_BUDGET_GB") o.memory_budget_bytes = (int64_t)(std::stod(v) * 1e9);
        else std::cout << "Unknown parameter: " << k << ", skipping..." << std::endl;
        line_num++;
    }
    C.phytree = trim(C.phytree, " \"\t\n");
    C.align = trim(C.align, " \"\t\n");
    C.output = trim(C.output, " \"\t\n");
    C.segment = trim(C.segment, " \"\t\n");
    C.o.init_lrate2 = (C.o.hyper_lrate2_a == 0) ? 0 : lrate2_init;  // main.cpp:286
    return C;
}

// ---------------------------------------------------------------------------
// SAMPLE_HYPER: the hyper-parameter MH between chains (BPP::sample_hyperparam,
// bpp.cpp:324-477) on the host.  Its draws come from the model's own
// generator, seeded with SEED (bpp.hpp:177-178): here a Philox4x32-10 word
// stream from SEED (Salmon et al., SC'11), the same stream layout and
// samplers as the chains' (uniform (w + 0.5) 2^-32, Box-Muller normal,
// Marsaglia-Tsang gamma with the a < 1 boost).
// ---------------------------------------------------------------------------
struct HostStream {
    uint32_t seed = 0;
    uint64_t pos = 0, blk = ~0ull;
    uint32_t cache[4] = {0, 0, 0, 0};
    uint32_t word() {
        const uint64_t b = pos >> 2;
        if (b != blk) {
            uint32_t c0 = (uint32_t)b, c1 = (uint32_t)(b >> 32), c2 = 0, c3 = 0, k0 = seed, k1 = 0;
            for (int r = 0; r < 10; r++) {
                const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
                const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
                c1 = (uint32_t)p1; c3 = (uint32_t)p0; c0 = n0; c2 = n2;
                k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
            }
            cache[0] = c0; cache[1] = c1; cache[2] = c2; cache[3] = c3;
            blk = b;
        }
        return cache[pos++ & 3];
    }
    double uniform() { return ((double)word() + 0.5) * 2.3283064365386963e-10; }
    double normal() {
        const double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
    double gamma(double a, double b) {
        if (a < 1.0) {
            const double g = gamma(a + 1.0, 1.0);
            const double u = uniform();
            return b * g * std::pow(u, 1.0 / a);
        }
        const double d = a - 1.0 / 3.0, c = 1.0 / std::sqrt(9.0 * d);
        double x, v;
        for (;;) {
            do {
                x = normal();
                v = 1.0 + c * x;
            } while (v <= 0.0);
            v = v * v * v;
            const double u = uniform(), x2 = x * x;
            if (u < 1.0 - 0.0331 * x2 * x2) break;
            if (std::log(u) < 0.5 * x2 + d * (1.0 - v + std::log(v))) break;
        }
        return b * d * v;
    }
};

static double gamma_density(double x, double a, double b) {   // the Gamma(a, scale b) density
    if (x < 0) return 0.0;
    if (x == 0) return (a == 1) ? 1.0 / b : 0.0;
    return std::exp((a - 1) * std::log(x) - x / b - std::lgamma(a) - a * std::log(b));
}
static double ln_beta(double a, double b) { return std::lgamma(a) + std::lgamma(b) - std::lgamma(a + b); }

// h: nprior_a, nprior_b, cprior_a, cprior_b, prior_l_a, prior_l_b, prior_g_a,
// prior_g_b, prior_l2_a, prior_l2_b.  rates: [n][5] n, c, g, l, l2 of every
// element of the run (in id order; filtered elements with their start values).
static void sample_hyperparam(HostStream& rng, double* h, const vector<double>& rates, int n) {
    const double p = 1, r = 1, q = 0.1, s = 0.1, ne = (double)n;
    const double vna = 100, vnb = 100, vca = 100, vcb = 100;
    const double nap = rng.gamma(vna, h[0] / vna);
    const double cap = rng.gamma(vca, h[2] / vca);
    const double nbp = rng.gamma(vnb, h[1] / vnb);
    const double cbp = rng.gamma(vcb, h[3] / vcb);
    auto shape_scale = [&](int col, double ap, double bp, double& a, double& b, double va, double vb) {
        double sum_r = 0, lpr = 0;
        for (int e = 0; e < n; e++) {
            sum_r += rates[(size_t)e * 5 + col];
            lpr += std::log(rates[(size_t)e * 5 + col]);
        }
        double mr = (ap - 1) * (std::log(p) + lpr) - (q + sum_r) / bp - (ne + r) * std::lgamma(ap) -
                    std::log(bp) * ap * (s + ne);
        mr -= (a - 1) * (std::log(p) + lpr) - (q + sum_r) / b - (ne + r) * std::lgamma(a) - std::log(b) * a * (s + ne);
        const double hr = std::log(gamma_density(a, va, ap / va)) - std::log(gamma_density(ap, va, a / va)) +
                          std::log(gamma_density(b, vb, bp / vb)) - std::log(gamma_density(bp, vb, b / vb));
        if (std::log(rng.uniform()) < mr + hr) { a = ap; b = bp; }
    };
    shape_scale(0, nap, nbp, h[0], h[1], vna, vnb);   // accelerated-rate prior
    shape_scale(1, cap, cbp, h[2], h[3], vca, vcb);   // conserved-rate prior
    auto beta_pair = [&](int col, double& a, double& b) {
        double u = rng.uniform() * (1.3 - 0.7) + 0.7;
        const double ap = a * u;
        u = rng.uniform() * (1.3 - 0.7) + 0.7;
        const double bp = b * u;
        double log_p = 0, log_pc = 0;
        for (int e = 0; e < n; e++) {
            log_p += std::log(rates[(size_t)e * 5 + col]);
            log_pc += std::log(1 - rates[(size_t)e * 5 + col]);
        }
        double mr = (ap - a) * (log_p - 1) + (bp - b) * (log_pc - 1);
        mr += ne * (ln_beta(a, b) - ln_beta(ap, bp));
        const double hr = std::log(a) - std::log(ap) + std::log(b) - std::log(bp);
        if (std::log(rng.uniform()) < mr + hr) { a = ap; b = bp; }
    };
    beta_pair(3, h[4], h[5]);   // l
    beta_pair(4, h[8], h[9]);   // l2
    beta_pair(2, h[6], h[7]);   // g
}

int main(int argc, char** argv) {
    auto t_start = std::chrono::steady_clock::now();
    std::cout << std::fixed << std::setprecision(4);
    if (argc < 2) die("Please specify the path of the parameter file.");
    Config C = load_config(argv[1]);
    if (!dir_exists(C.output)) {
        std::cout << "output path doesn't exist or empty!" << std::endl;
        return 1;
    }
    if (C.chain > 1 && !C.sample_hyper && C.o.precision != PACC_FP64 && C.o.precision != PACC_FP32)
        die("CHAIN > 1: a later chain needs GPU_PRECISION fp64 or fp32");
    Profile prof = load_profile(C.align, C.segment);
    Tree T;
    double pi[4], Q[16];
    load_mod(C.phytree, T, pi, Q);
    const int S = T.S, N = 2 * S - 1;
    // MatchProfAndTree (bpp.cpp:133-184)
    vector<int> reorder(S, -1);
    bool matched = (int)prof.names.size() >= S;
    for (int s = 0; s < S && matched; s++) {
        auto it = std::find(prof.names.begin(), prof.names.end(), T.names[s]);
        if (it == prof.names.end()) matched = false;
        else reorder[s] = (int)(it - prof.names.begin());
    }
    vector<string> X(S);
    vector<string> species_names(S);
    if (matched) {
        std::cout << "The species in profile and tree match perfectly. Reorder the species in profile matrix by the tree."
                  << std::endl;
        for (int s = 0; s < S; s++) { X[s] = prof.X[reorder[s]]; species_names[s] = T.names[s]; }
    } else {
        std::cout << "The species in phylogenetic profile and tree cannot be matched literally; using the order of the data."
                  << std::endl;
        if ((int)prof.X.size() < S) die("(Error. Fewer sequences than tree leaves)");
        for (int s = 0; s < S; s++) { X[s] = prof.X[s]; species_names[s] = prof.names[s]; }
    }
    vector<int> outgroup = species_ids(C.outgroup, species_names);
    vector<int> conserve = species_ids(C.conserve, species_names);
    pacc_model model;
    model.n_species = S;
    model.children = T.children.data();
    model.distances = T.distances.data();
    model.pi = pi;
    model.rate_matrix = Q;
    model.outgroup = outgroup.data();
    model.n_outgroup = (int)outgroup.size();
    model.conserve = conserve.data();
    model.n_conserve = (int)conserve.size();
    const int Cn = (int)prof.elem_names.size();
    vector<long> el_start(Cn), el_len(Cn);
    {
        long start = 0;
        for (int c = 0; c < Cn; c++) {
            long len = prof.pos[c].second - prof.pos[c].first;
            el_start[c] = start;
            el_len[c] = len;
            start += len;  // consecutive elements (bpp.hpp:257-274)
        }
    }
    // ids (main.cpp:406-440)
    vector<int> ids;
    if (C.id_path.empty()) {
        if (C.batch == -1) for (int c = 0; c < Cn; c++) ids.push_back(c);
        else {
            int tmp = (int)std::ceil(Cn / 3);
            for (int c = C.batch * tmp; c < (C.batch + 1) * tmp && c < Cn; c++) ids.push_back(c);
        }
    } else {
        std::ifstream in(C.id_path.c_str());
        if (!in) die("Cannot open the id file: " + C.id_path);
        string line;
        while (std::getline(in, line)) {
            std::istringstream ls(line);
            string tk;
            ls >> tk;
            tk = trim(tk);
            if (tk.empty()) continue;
            ids.push_back(std::atoi(tk.c_str()));
        }
    }
    std::cout << ids.size() << " of elements to be computed" << std::endl;
    const string out = C.output + "/" + C.prefix;
    {
        std::ofstream h((out + "_hyper.txt").c_str());
        h << "iter\tnprior_a\tnprior_b\tcprior_a\tcprior_b\tprior_l_a\tprior_l_b\tprior_g_a\tprior_g_b\n";
        h << 0 << "\t" << C.o.acce_prior_a << "\t" << C.o.acce_prior_b << "\t" << C.o.conserve_prior_a << "\t"
          << C.o.conserve_prior_b << "\t" << C.o.hyper_lrate_a << "\t" << C.o.hyper_lrate_b << "\t" << C.o.hyper_grate_a
          << "\t" << C.o.hyper_grate_b << std::endl;
        std::ofstream sp((out + "_species_names.txt").c_str());
        for (int s = 0; s < N; s++) sp << T.names[s] << std::endl;
    }
    const string zpath[3] = {out + "_rate_postZ_M0.txt", out + "_rate_postZ_M1.txt", out + "_rate_postZ_M2.txt"};
    std::ofstream oz[3];
    for (int m = 0; m < 3; m++) {
        oz[m].open(zpath[m].c_str());
        oz[m] << "No.\tn_rate\tc_rate\tg_rate\tl_rate\tl2_rate";
        for (int s = 0; s < N; s++)
            for (int k = 0; k < 4; k++) oz[m] << "\t" << T.names[s] << "_" << k;
        oz[m] << std::endl;
    }
    const int Tn = C.o.burnin + C.o.mcmc;
    if (C.verbose) C.o.trace_iters = Tn;
    // CHAIN has no default in PhyloAcc-ST (main.cpp:57): with CHAIN < 1 no
    // chain runs and only the headers above are written (main.cpp:445-509)
    // batch of elements in tree leaf order
    vector<int64_t> no(ids.size());
    vector<int32_t> lens(ids.size());
    vector<int64_t> offs(ids.size());
    vector<uint8_t> bases;
    for (size_t i = 0; i < ids.size(); i++) {
        int c = ids[i];
        if (c < 0 || c >= Cn) die("element id out of range");
        no[i] = c;
        lens[i] = (int32_t)el_len[c];
        offs[i] = (int64_t)bases.size();
        for (int s = 0; s < S; s++) {
            const string& row = X[s];
            for (long g = 0; g < el_len[c]; g++) {
                long p = el_start[c] + g;
                bases.push_back(p < (long)row.size() ? (uint8_t)row[p] : (uint8_t)0);
            }
        }
    }
    vector<pacc_result> res(ids.size());
    vector<int32_t> maxz(ids.size() * 3 * N);
    vector<double> postz(ids.size() * 3 * N * 4);
    const int TI = C.o.trace_iters;
    vector<double> tr((size_t)ids.size() * 6 * 3 * std::max(TI, 1));
    vector<int8_t> trz((size_t)ids.size() * 3 * std::max(TI, 1) * N);
    pacc_element_batch batch;
    batch.n_elements = (int32_t)ids.size();
    batch.element_no = no.data();
    batch.lengths = lens.data();
    batch.offsets = offs.data();
    batch.bases = bases.data();
    double kernel_ms = 0;
    // SAMPLE_HYPER (main.cpp:466-509): only M2 runs, each chain from the state
    // the previous one left (bpp_c.cpp:148-177,475-485); the hyper-parameters
    // are drawn between chains; _elem_lik.txt gets (loglik_all, loglik_Max)
    // rows per chain (bpp.cpp:622-634) and no _elem_Z files are written.
    const bool hyp = C.sample_hyper;
    C.o.sample_hyper = hyp ? 1 : 0;
    double hyper[10] = {C.o.acce_prior_a, C.o.acce_prior_b, C.o.conserve_prior_a, C.o.conserve_prior_b,
                        C.o.hyper_lrate_a, C.o.hyper_lrate_b, C.o.hyper_grate_a, C.o.hyper_grate_b,
                        C.o.hyper_lrate2_a, C.o.hyper_lrate2_b};
    HostStream hyper_rng;
    hyper_rng.seed = C.o.seed;
    vector<int8_t> state_z, end_z;
    vector<double> state_rates;
    if (hyp) {
        end_z.assign(ids.size() * N, 0);
        state_rates.resize(ids.size() * 5);
        for (size_t i = 0; i < ids.size(); i++) {   // bpp.cpp:215-220
            const double v[5] = {C.o.init_acce_rate, C.o.init_conserve_rate, C.o.init_grate, C.o.init_lrate,
                                 C.o.init_lrate2};
            for (int q = 0; q < 5; q++) state_rates[i * 5 + q] = v[q];
        }
        std::ofstream ol((out + "_elem_lik.txt").c_str());
        ol << "No.\tID\tloglik_all\tloglik_Max" << std::endl;
    }
    // CHAIN chains (main.cpp:445): each runs every element from SEED; without
    // SAMPLE_HYPER a later chain starts from Z = 0 (bpp_c.cpp:148-151).
    // _rate_postZ rows and traces are appended per chain, _elem_lik / _elem_Z
    // are the last chain's.
    for (int chain = 0; chain < C.chain; chain++) {
        C.o.chain = hyp ? 0 : chain;
        if (hyp) {
            C.o.acce_prior_a = hyper[0]; C.o.acce_prior_b = hyper[1];
            C.o.conserve_prior_a = hyper[2]; C.o.conserve_prior_b = hyper[3];
            C.o.hyper_lrate_a = hyper[4]; C.o.hyper_lrate_b = hyper[5];
            C.o.hyper_grate_a = hyper[6]; C.o.hyper_grate_b = hyper[7];
            C.o.hyper_lrate2_a = hyper[8]; C.o.hyper_lrate2_b = hyper[9];
            batch.start_z = chain > 0 ? state_z.data() : nullptr;
            batch.start_rates = state_rates.data();
        }
        int st = 0;
        pacc_ctx* ctx = pacc_create(&model, &C.o, &st);
        if (!ctx) die(string("pacc_create failed: ") + pacc_last_error(nullptr));
        for (size_t i = 0; i < ids.size(); i++) {
            std::memset(&res[i], 0, sizeof(pacc_result));
            res[i].max_z = &maxz[i * 3 * N];
            res[i].post_z = &postz[i * 3 * N * 4];
            if (hyp) res[i].end_z = &end_z[i * N];
            if (TI > 0) {
                double* b = &tr[i * 6 * 3 * TI];
                res[i].trace.loglik = b;
                res[i].trace.n_rate = b + 3 * TI;
                res[i].trace.c_rate = b + 6 * TI;
                res[i].trace.g_rate = b + 9 * TI;
                res[i].trace.l_rate = b + 12 * TI;
                res[i].trace.l2_rate = b + 15 * TI;
                res[i].trace.z = &trz[i * 3 * TI * N];
            }
        }
        if (!ids.empty()) {
            st = pacc_run(ctx, &batch, res.data());
            if (st != PACC_OK) die(string("GPU run failed: ") + pacc_last_error(ctx));
        }
        // rate_postZ rows (bpp_c2.cpp:774-784), model files M0, M1 (resZ 2), M2 (resZ 1)
        for (size_t i = 0; i < ids.size(); i++) {
            const pacc_result& r = res[i];
            if (r.status == PACC_FILTERED || r.status == PACC_SAMPLER_ERROR) continue;
            for (int m = hyp ? 2 : 0; m < 3; m++) {
                const pacc_model_result& mr = r.model[m];
                oz[m] << r.element_no << "\t" << mr.n_rate << "\t" << mr.c_rate << "\t" << mr.g_rate << "\t"
                      << mr.l_rate << "\t" << mr.l2_rate;
                for (int s = 0; s < N; s++)
                    for (int k = 0; k < 4; k++) oz[m] << "\t" << postz[(i * 3 + m) * N * 4 + s * 4 + k];
                oz[m] << std::endl;
                if (C.verbose || mr.failure) {
                    // Output_sampling (bpp_c2.cpp:706-736): header with the first chain,
                    // later chains appended
                    const string path = out + "_mcmc_trace_M" + std::to_string(m) + "_" +
                                        std::to_string(r.element_no) + ".txt";
                    std::ofstream tf(path.c_str(), chain == 0 ? std::ios::out : std::ios::app);
                    tf.precision(8);
                    if (chain == 0) {
                        tf << "loglik\trate_n\trate_c\tgrate\tlrate\tlrate2\t";
                        for (int s = 0; s < N; s++) tf << T.names[s] << "\t";
                        tf << std::endl;
                    }
                    const double* b = &tr[i * 6 * 3 * TI];
                    for (int it = 0; it < TI; it++) {
                        for (int q = 0; q < 6; q++) tf << b[q * 3 * TI + m * TI + it] << "\t";
                        for (int s = 0; s < N; s++) tf << (int)trz[((i * 3 + m) * TI + it) * N + s] << "\t";
                        tf << std::endl;
                    }
                }
            }
        }
        pacc_counters pc;
        pacc_get_counters(ctx, &pc);
        kernel_ms += pc.kernel_ms;
        pacc_destroy(ctx);
        if (hyp) {
            // the chains' end states become the next start (elements that did
            // not run keep theirs), then the hyper-parameter MH and the rows
            if (state_z.empty()) state_z.assign(ids.size() * N, -128);
            for (size_t i = 0; i < ids.size(); i++) {
                if (res[i].status == PACC_FILTERED || res[i].status == PACC_SAMPLER_ERROR) continue;
                std::memcpy(&state_z[i * N], &end_z[i * N], N);
                for (int q = 0; q < 5; q++) state_rates[i * 5 + q] = res[i].end_rates[q];
            }
            sample_hyperparam(hyper_rng, hyper, state_rates, (int)ids.size());
            std::ofstream h((out + "_hyper.txt").c_str(), std::ios::app);
            h << chain;
            for (int q = 0; q < 10; q++) h << "\t" << hyper[q];
            h << std::endl;
            std::ofstream ol((out + "_elem_lik.txt").c_str(), std::ios::app);
            ol.precision(8);
            for (size_t i = 0; i < ids.size(); i++)
                ol << ids[i] << "\t" << prof.elem_names[ids[i]] << "\t" << res[i].model[2].loglik << "\t"
                   << res[i].model[2].max_loglik << std::endl;
        }
    }
    // _elem_lik.txt and _M*_elem_Z.txt (bpp.cpp:568-619)
    if (!hyp && C.chain >= 1) {
        std::ofstream ol((out + "_elem_lik.txt").c_str());
        ol.precision(8);
        ol << "No.\tID\tloglik_Null\tloglik_Acc\tloglik_Full\tlogBF1\tlogBF2\tloglik_Max_M0\tloglik_Max_M1\tloglik_Max_M2"
           << std::endl;
        for (size_t i = 0; i < ids.size(); i++) {
            const pacc_result& r = res[i];
            int c = ids[i];
            double null_ = r.model[0].loglik, acc = r.model[1].loglik, full = r.model[2].loglik;
            ol << c << "\t" << prof.elem_names[c] << "\t" << null_ << "\t" << acc << "\t" << full << "\t";
            ol << acc - null_ << "\t" << acc - full;
            ol << "\t" << r.model[0].max_loglik << "\t" << r.model[1].max_loglik << "\t" << r.model[2].max_loglik;
            ol << std::endl;
        }
        for (int m = 0; m < 3; m++) {
            std::ofstream ozz((out + "_M" + std::to_string(m) + "_elem_Z.txt").c_str());
            ozz << "No.";
            for (int s = 0; s < N; s++) ozz << "\t" << T.names[s];
            ozz << std::endl;
            for (size_t i = 0; i < ids.size(); i++) {
                ozz << ids[i];
                for (int s = 0; s < N; s++) ozz << "\t" << maxz[(i * 3 + m) * N + s];
                ozz << std::endl;
            }
        }
    }
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    std::cout << "\n\ntime used:  " << (long)(secs / 60) << " min. (" << secs << " s; GPU kernel "
              << kernel_ms / 1000.0 << " s)" << std::endl;
    return 0;
}
