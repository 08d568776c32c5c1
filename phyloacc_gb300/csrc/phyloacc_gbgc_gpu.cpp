// phyloacc-gbgc-gpu — drop-in replacement for the PhyloAcc-ST-GBGC executable
// (the gBGC model, src/PhyloAcc-ST-GBGC/SRC).
//
//     phyloacc-gbgc-gpu <config file>
//
// Reads the same key-value configuration (main.cpp:83-259), the same inputs
// (.mod tree + rate matrix, FASTA alignment, bed segments, optional id list)
// and writes the same tables (main.cpp:296-323, bpp_c2.cpp:567-660,
// bpp.cpp:536-574):
//   <PREFIX>_elem_lik.txt, <PREFIX>_1_elem_Z.txt, <PREFIX>_rate_postZ_{0,1,2}.txt,
//   <PREFIX>_hyper.txt, <PREFIX>_species_names.txt and, with VERBOSE,
//   <PREFIX>_mcmc_trace_{0,1,2}_{No}.txt.
// The chains run on the GPU through pacc_gbgc_run (include/pacc.h).
// Extra keys (ignored by the reference): GPU_PRECISION fp64|fp32, GPU_DEVICE,
// GPU_MEMORY_BUDGET_GB (device memory for the traces of one launch).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iomanip>

#include "pacc.h"
#include "cli_io.h"

struct GConfig {
    string phytree, align, segment, id_path, output, prefix = "test";
    string outgroup, target, conserve;
    int batch = 0, chain = 0, indel = 0;
    bool verbose = true, sample_hyper = false;
    pacc_gbgc_opts g;
    pacc_opts o;
};

static GConfig load_config(const string& path) {
    GConfig C;
    pacc_gbgc_default_opts(&C.g);
    pacc_default_opts(&C.o);
    C.o.precision = PACC_FP64;
    std::ifstream in(path.c_str());
    if (!in) die("Cannot open the parameters file: " + path);
    string line;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        string k, v;
        ls >> k;
        if (k.empty() || k[0] == '#') continue;
        ls >> v;
        pacc_gbgc_opts& g = C.g;
        if (k == "PHYTREE_FILE") C.phytree = v;
        else if (k == "ALIGN_FILE") C.align = v;
        else if (k == "SEG_FILE") C.segment = v;
        else if (k == "ID_FILE") C.id_path = v;
        else if (k == "BATCH") C.batch = std::stoi(v);
        else if (k == "RESULT_FOLDER") C.output = v;
        else if (k == "PREFIX") C.prefix = v;
        else if (k == "SEED") g.seed = (uint32_t)std::stoi(v);
        else if (k == "CONSERVE_RATE") g.conserve_rate = std::stod(v);
        else if (k == "ACCE_RATE") g.acce_rate = std::stod(v);
        else if (k == "CONSERVE_PRIOR_A") g.conserve_prior_a = std::stod(v);
        else if (k == "CONSERVE_PRIOR_B") g.conserve_prior_b = std::stod(v);
        else if (k == "ACCE_PRIOR_A") g.acce_prior_a = std::stod(v);
        else if (k == "ACCE_PRIOR_B") g.acce_prior_b = std::stod(v);
        else if (k == "BURNIN") g.burnin = std::stoi(v);
        else if (k == "MCMC") g.mcmc = std::stoi(v);
        else if (k == "PREP_LRATE") g.prep_lrate = std::stod(v);
        else if (k == "PREP_GRATE") g.prep_grate = std::stod(v);
        else if (k == "CHAIN") C.chain = std::stoi(v);
        else if (k == "OUTGROUP") C.outgroup = v;
        else if (k == "TARGETSPECIES") C.target = v;
        else if (k == "CONSERVE") C.conserve = v;
        else if (k == "CONSERVE_PROP") g.conserve_prop = std::stod(v);
        else if (k == "GAP_PROP") g.missing_thres = std::stod(v);
        else if (k == "CONSTOMIS") g.cons_to_mis = std::stod(v);
        else if (k == "GAPCHAR") g.gapchar = v.empty() ? '*' : v[0];
        else if (k == "INDEL") C.indel = std::stoi(v);
        else if (k == "SAMPLE_HYPER") C.sample_hyper = v == "1" || v == "true";
        else if (k == "VERBOSE") C.verbose = v == "1" || v == "true";
        else if (k == "ROPT" || k == "CUB" || k == "NLB" || k == "ADAPT_FREQ" || k == "REF" || k == "INDEL2" ||
                 k == "SAMPLE_INDEL" || k == "NUM_THREAD" || k == "RESULT_INDIV") {}
        else if (k == "GPU_PRECISION") C.o.precision = (v == "fp32" || v == "FP32") ? PACC_FP32 : PACC_FP64;
        else if (k == "GPU_DEVICE") C.o.device = std::stoi(v);
        else if (k == "GPU_MEMORY_BUDGET_GB") C.o.memory_budget_bytes = (int64_t)(std::stod(v) * 1e9);
        else std::cout << "Unknown parameter: " << k << ", skipping..." << std::endl;
    }
    C.phytree = trim(C.phytree, " \"\t\n");
    C.align = trim(C.align, " \"\t\n");
    C.output = trim(C.output, " \"\t\n");
    C.segment = trim(C.segment, " \"\t\n");
    return C;
}

int main(int argc, char** argv) {
    auto t_start = std::chrono::steady_clock::now();
    if (argc < 2) die("Please specify the path of the parameter file.");
    GConfig C = load_config(argv[1]);
    if (!dir_exists(C.output)) {
        std::cout << "output path doesn't exist or empty!" << std::endl;
        return 1;
    }
    if (C.indel > 0) die("INDEL > 0 (the five-state model) is not supported");
    if (C.sample_hyper) die("SAMPLE_HYPER is not supported for the gBGC model");
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
    vector<string> X(S), species_names(S);
    if (matched) {
        for (int s = 0; s < S; s++) { X[s] = prof.X[reorder[s]]; species_names[s] = T.names[s]; }
    } else {
        if ((int)prof.X.size() < S) die("(Error. Fewer sequences than tree leaves)");
        for (int s = 0; s < S; s++) { X[s] = prof.X[s]; species_names[s] = prof.names[s]; }
    }
    vector<int> outgroup = species_ids(C.outgroup, species_names);
    vector<int> conserve = species_ids(C.conserve, species_names);
    vector<int> target = species_ids(C.target, species_names);
    C.g.target = target.data();
    C.g.n_target = (int)target.size();
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
            el_len[c] = prof.pos[c].second - prof.pos[c].first;
            el_start[c] = start;
            start += el_len[c];
        }
    }
    // ids (main.cpp:327-370): BATCH 0 runs every element
    vector<int> ids;
    if (C.id_path.empty()) {
        if (C.batch == 0) for (int c = 0; c < Cn; c++) ids.push_back(c);
        else {
            const int tmp = Cn / 3;
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
            if (!tk.empty()) ids.push_back(std::atoi(tk.c_str()));
        }
    }
    std::cout << ids.size() << " of elements to be computed" << std::endl;
    const string out = C.output + "/" + C.prefix;
    std::ofstream oz[3];
    for (int m = 0; m < 3; m++) {
        oz[m].open((out + "_rate_postZ_" + std::to_string(m) + ".txt").c_str());
        oz[m] << "No.\tn_rate\tc_rate\tgBC";
        for (int s = 0; s < N; s++) oz[m] << "\t" << T.names[s] << "_B";
        for (int s = 0; s < N; s++)
            for (int k = 0; k < 4; k++) oz[m] << "\t" << T.names[s] << "_" << k;
        oz[m] << std::endl;
    }
    {
        std::ofstream sp((out + "_species_names.txt").c_str());
        for (int s = 0; s < N; s++) sp << T.names[s] << std::endl;
    }
    std::ofstream oh((out + "_hyper.txt").c_str());
    oh << "iter\tnprior_a\tnprior_b\tcprior_a\tcprior_b\tindel\tindel2\tgrate\tlrate\n";
    // the batch of elements in tree leaf order
    vector<int64_t> no(ids.size());
    vector<int32_t> lens(ids.size());
    vector<int64_t> offs(ids.size());
    vector<uint8_t> bases;
    for (size_t i = 0; i < ids.size(); i++) {
        const int c = ids[i];
        if (c < 0 || c >= Cn) die("element id out of range");
        no[i] = c;
        lens[i] = (int32_t)el_len[c];
        offs[i] = (int64_t)bases.size();
        for (int s = 0; s < S; s++)
            for (long g = 0; g < el_len[c]; g++) {
                const long p = el_start[c] + g;
                bases.push_back(p < (long)X[s].size() ? (uint8_t)X[s][p] : (uint8_t)0);
            }
    }
    pacc_element_batch batch;
    std::memset(&batch, 0, sizeof(batch));
    batch.n_elements = (int32_t)ids.size();
    batch.element_no = no.data();
    batch.lengths = lens.data();
    batch.offsets = offs.data();
    batch.bases = bases.data();
    const int TT = C.g.burnin + C.g.mcmc;
    vector<pacc_gbgc_result> res(ids.size());
    vector<int32_t> maxz(ids.size() * 3 * N);
    vector<int8_t> maxb(ids.size() * 3 * N);
    vector<double> postb(ids.size() * 3 * N), postz(ids.size() * 3 * N * 4);
    vector<double> tr(C.verbose ? ids.size() * 3 * (size_t)TT * (4 + 2 * N) : 0);
    // per element over all chains: the last chain's values (BPP's vectors,
    // zero for elements not run)
    vector<double> ll_null(Cn, 0), ll_res(Cn, 0), ll_all(Cn, 0), ll_max[3];
    vector<vector<int>> elem_z(Cn, vector<int>(N, 0));
    for (int m = 0; m < 3; m++) ll_max[m].assign(Cn, 0);
    double kernel_ms = 0;
    int st = 0;
    pacc_ctx* ctx = nullptr;
    for (int chain = 0; chain < C.chain; chain++) {
        // sample_proposal's hyper row (bpp.cpp:224-252): the starting values
        oh << chain << "\t" << C.g.acce_prior_a << "\t" << C.g.acce_prior_b << "\t" << C.g.conserve_prior_a << "\t"
           << C.g.conserve_prior_b << "\t" << 0 << "\t" << 0 << "\t" << C.g.prep_grate << "\t" << C.g.prep_lrate
           << std::endl;
        C.g.chain = chain;
        if (!ctx) {
            ctx = pacc_create(&model, &C.o, &st);
            if (!ctx) die(string("pacc_create failed: ") + pacc_last_error(nullptr));
        }
        for (size_t i = 0; i < ids.size(); i++) {
            std::memset(&res[i], 0, sizeof(pacc_gbgc_result));
            res[i].max_z = &maxz[i * 3 * N];
            res[i].max_b = &maxb[i * 3 * N];
            res[i].post_b = &postb[i * 3 * N];
            res[i].post_z = &postz[i * 3 * N * 4];
            if (C.verbose) res[i].trace = &tr[i * 3 * (size_t)TT * (4 + 2 * N)];
        }
        if (!ids.empty()) {
            st = pacc_gbgc_run(ctx, &C.g, &batch, res.data());
            if (st != PACC_OK) die(string("GPU run failed: ") + pacc_last_error(ctx));
        }
        for (size_t i = 0; i < ids.size(); i++) {
            const pacc_gbgc_result& r = res[i];
            if (r.status != PACC_OK) continue;
            const int c = ids[i];
            // Output_init per model, M0, M2, M1 as they finish (bpp_c2.cpp:603-660)
            const int order[3] = {0, 2, 1};
            for (int q = 0; q < 3; q++) {
                const int m = order[q];
                if (C.verbose) {
                    // Output_sampling (bpp_c2.cpp:567-600)
                    const string path = out + "_mcmc_trace_" + std::to_string(m) + "_" + std::to_string(c) + ".txt";
                    std::ofstream tf(path.c_str(), chain == 0 ? std::ios::out : std::ios::app);
                    tf.precision(8);
                    if (chain == 0) {
                        tf << "loglik\trate_n\trate_c\tGB\t";
                        for (int s = 0; s < N; s++) tf << T.names[s] << "_B\t";
                        for (int s = 0; s < N; s++) tf << T.names[s] << "\t";
                        tf << std::endl;
                    }
                    const double* b = &tr[(i * 3 + m) * (size_t)TT * (4 + 2 * N)];
                    for (int it = 0; it < TT; it++) {
                        const double* row = b + (size_t)it * (4 + 2 * N);
                        tf << row[0] << "\t" << row[1] << "\t" << row[2] << "\t" << row[3] << "\t";
                        for (int s = 0; s < N; s++) tf << (int)row[4 + s] << "\t";
                        for (int s = 0; s < N; s++) tf << (int)row[4 + N + s] << "\t";
                        tf << std::endl;
                    }
                }
                oz[m] << c << "\t" << r.rates[m][0] << "\t" << r.rates[m][1] << "\t" << r.rates[m][2];
                for (int s = 0; s < N; s++) oz[m] << "\t" << postb[(i * 3 + m) * N + s];
                for (int s = 0; s < N; s++)
                    for (int k = 0; k < 4; k++) oz[m] << "\t" << postz[((i * 3 + m) * N + s) * 4 + k];
                oz[m] << std::endl;
            }
            ll_null[c] = r.loglik_null;
            ll_res[c] = r.loglik_res;
            ll_all[c] = r.loglik_all;
            for (int m = 0; m < 3; m++) ll_max[m][c] = r.max_loglik[m];
            for (int s = 0; s < N; s++) elem_z[c][s] = maxz[(i * 3 + 1) * N + s];
        }
        pacc_counters pc;
        pacc_get_counters(ctx, &pc);
        kernel_ms = pc.kernel_ms;
    }
    if (ctx) pacc_destroy(ctx);
    // BPP::Output_init (bpp.cpp:536-574): every element of the bed
    if (C.chain >= 1) {
        std::ofstream ol((out + "_elem_lik.txt").c_str());
        ol.precision(8);
        ol << "No.\tID\tloglik_NUll\tloglik_RES\tloglik_all\tlog_ratio\tloglik_Max1\tloglik_Max2\tloglik_Max3" << std::endl;
        for (int c = 0; c < Cn; c++) {
            ol << c << "\t" << prof.elem_names[c] << "\t" << ll_null[c] << "\t" << ll_res[c] << "\t" << ll_all[c] << "\t"
               << ll_res[c] - ll_null[c];
            for (int m = 0; m < 3; m++) ol << "\t" << ll_max[m][c];
            ol << std::endl;
        }
        std::ofstream ozz((out + "_1_elem_Z.txt").c_str());
        for (int s = 0; s < N; s++) ozz << T.names[s] << "_B\t";
        for (int s = 0; s < N; s++) ozz << T.names[s] << "\t";
        ozz << std::endl;
        for (int c = 0; c < Cn; c++) {
            for (int s = 0; s < N; s++) ozz << elem_z[c][s] << "\t";
            ozz << std::endl;
        }
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    std::cout << "\n\ntime used:  " << (long)(secs / 60) << " min. (" << secs << " s; GPU kernel "
              << kernel_ms / 1000.0 << " s)" << std::endl;
    return 0;
}
