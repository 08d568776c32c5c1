// oracle_st.cpp — TEST INFRASTRUCTURE (the oracle), never product code.
//
// A CPU restatement of PhyloAcc-ST's per-element Bayesian MCMC, kept in the
// reference's log-space arithmetic and control flow so that it can check the
// GPU path draw for draw.  Only tests/, __graft_entry__.smoke() and bench.py's
// CPU baseline use it.  Every function cites the reference file:line it
// restates (paths relative to the PhyloAcc repository).
//
// Deliberate replacements (the reference's third-party libraries are absent):
//   * GSL mt19937 + gsl_ran_* -> oracle_rng.h (same stream structure: one
//     sequential stream per element seeded with SEED, bpp_c.hpp:146-147);
//   * Armadillo eig_gen/inv   -> phyloacc_gb300/csrc/eigen4.h;
//   * gsl_ran_gamma_pdf       -> the Gamma density formula (log taken as in the reference);
//   * gsl_sf_lnbeta           -> lgamma(a) + lgamma(b) - lgamma(a+b).
// Parity of this file with the unmodified reference sources is checked by
// building those sources against stand-ins for the GSL/Armadillo subset they
// call (oracle/shim, oracle/Makefile) and comparing outputs.
#include "../include/pacc.h"
#include "oracle_rng.h"
#include "../phyloacc_gb300/csrc/eigen4.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double LOG_ZERO = -INFINITY;
const int K = 4;  // num_base: INDEL == 0 (bpp.hpp:247-253)

struct Mat4 { double a[4][4]; };
struct Mat3 { double a[3][3]; };
struct Vec4 { double v[4]; };

// Gamma(shape a, scale b) density, the quantity gsl_ran_gamma_pdf returns.
double gamma_pdf(double x, double a, double b) {
    if (x < 0) return 0.0;
    if (x == 0) return (a == 1) ? 1.0 / b : 0.0;
    return std::exp((a - 1) * std::log(x) - x / b - std::lgamma(a) - a * std::log(b));
}

// The reference always takes log(gsl_ran_gamma_pdf(...)) (bpp_c.cpp:784,801,1046-1047).
double log_gamma_pdf(double x, double a, double b) { return std::log(gamma_pdf(x, a, b)); }

double lnbeta(double a, double b) { return std::lgamma(a) + std::lgamma(b) - std::lgamma(a + b); }

// ---------------------------------------------------------------------------
// BPP: shared model (bpp.hpp:42-404, bpp.cpp:40-129, 486-504)
// ---------------------------------------------------------------------------
struct Model {
    int S = 0, N = 0;
    std::vector<int> ch0, ch1, parent;
    std::vector<double> distances;
    double pi[4], log_pi[4];
    double eigenval[4];
    double eigenvec[4][4];  // V^T (bpp.hpp:361)
    double eigeninv[4][4];  // (V^T)^-1 (bpp.hpp:362)
    std::vector<Mat4> log_cache_TM_null;
    std::vector<int> conservedgroup, outgroup;
    std::set<int> upper, upper_conserve;
    pacc_opts o;
    std::string error;
};

// log P^T(d*r) = log(eigeninv * diag(exp(eigenval*d*r)) * eigenvec) (bpp.hpp:375-380)
Mat4 log_tm(const Model& M, double d, double r, bool scaled) {
    double e[4];
    for (int i = 0; i < K; i++) e[i] = std::exp(scaled ? M.eigenval[i] * d * r : M.eigenval[i] * d);
    Mat4 out;
    for (int a = 0; a < K; a++)
        for (int b = 0; b < K; b++) {
            double s = 0;
            for (int i = 0; i < K; i++) s += M.eigeninv[a][i] * (M.eigenvec[i][b] * e[i]);
            out.a[a][b] = std::log(s);
        }
    return out;
}

Mat4 log_identity() {  // bpp.hpp:390-391
    Mat4 m;
    for (int a = 0; a < K; a++)
        for (int b = 0; b < K; b++) m.a[a][b] = (a == b) ? 0.0 : LOG_ZERO;
    return m;
}

// BPP::log_multi (bpp.hpp:427-445): result[j] = log sum_i exp(log_x(i,j) + log_y[i])
Vec4 log_multi(const Mat4& lx, const Vec4& ly) {
    double t[4][4];
    double mx = LOG_ZERO;
    bool first = true;
    for (int j = 0; j < K; j++)        // Armadillo is column-major: scan column by column
        for (int i = 0; i < K; i++) {
            t[i][j] = lx.a[i][j] + ly.v[i];
            if (first || t[i][j] > mx) { mx = t[i][j]; first = false; }
        }
    Vec4 r;
    if (mx == LOG_ZERO) {
        for (int j = 0; j < K; j++) r.v[j] = LOG_ZERO;
        return r;
    }
    for (int j = 0; j < K; j++) {
        double s = 0;
        for (int i = 0; i < K; i++) s += std::exp(t[i][j] - mx);
        r.v[j] = std::log(s) + mx;
    }
    return r;
}

// BPP::log_exp_sum (bpp.hpp:471-479)
double log_exp_sum(const double* y, int n) {
    double mx = y[0];
    for (int i = 1; i < n; i++) if (y[i] > mx) mx = y[i];
    if (mx == LOG_ZERO) return LOG_ZERO;
    double s = 0;
    for (int i = 0; i < n; i++) s += std::exp(y[i] - mx);
    return std::log(s) + mx;
}

// BPP::log_sample (bpp.hpp:481-485)
void log_sample(const double* y, int n, double* out) {
    double mx = y[0];
    for (int i = 1; i < n; i++) if (y[i] > mx) mx = y[i];
    for (int i = 0; i < n; i++) out[i] = std::exp(y[i] - mx);
}

bool build_model(const pacc_model* pm, const pacc_opts* po, Model& M) {
    M.o = *po;
    M.S = pm->n_species;
    M.N = 2 * M.S - 1;
    int N = M.N;
    M.ch0.assign(N, -1); M.ch1.assign(N, -1); M.parent.assign(N, -1);
    M.distances.assign(pm->distances, pm->distances + N);
    // InitPhyloTree (bpp.cpp:98-117)
    for (int i = 0; i < N; i++) {
        M.ch0[i] = pm->children[2 * i];
        M.ch1[i] = pm->children[2 * i + 1];
        if (M.ch0[i] >= 0) M.parent[M.ch0[i]] = i;
        if (M.ch1[i] >= 0) M.parent[M.ch1[i]] = i;
    }
    for (int i = 0; i < K; i++) { M.pi[i] = pm->pi[i]; M.log_pi[i] = std::log(M.pi[i]); }
    // eig_gen / inv (bpp.hpp:357-362)
    double lam[4], V[16], Vi[16];
    if (pacc_eigen::decompose(4, pm->rate_matrix, lam, V, Vi) != pacc_eigen::EIG_OK) {
        M.error = "rate matrix eigendecomposition failed";
        return false;
    }
    for (int i = 0; i < 4; i++) {
        M.eigenval[i] = lam[i];
        for (int j = 0; j < 4; j++) {
            M.eigenvec[i][j] = V[j * 4 + i];  // V^T
        }
    }
    // eigeninv = inv(V^T) = (V^-1)^T
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) M.eigeninv[i][j] = Vi[j * 4 + i];
    // log_cache_TM_null (bpp.hpp:366-397); the root entry stays zero
    M.log_cache_TM_null.assign(N, Mat4{});
    for (int i = 0; i < N; i++)
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++) M.log_cache_TM_null[i].a[a][b] = 0.0;
    for (int i = 0; i < N - 1; i++) {
        if (M.distances[i] > 1e-10) M.log_cache_TM_null[i] = log_tm(M, M.distances[i], 1.0, false);
        else M.log_cache_TM_null[i] = log_identity();
    }
    M.outgroup.assign(pm->outgroup, pm->outgroup + pm->n_outgroup);
    M.conservedgroup.assign(pm->conserve, pm->conserve + pm->n_conserve);
    // getUppertree (bpp.cpp:486-504), bpp.hpp:309-310
    auto upper_of = [&](const std::vector<int>& grp, std::set<int>& out) {
        for (int p0 : grp) {
            int p = p0;
            while (p != N - 1) {
                out.insert(p);
                p = M.parent[p];
                if (p < 0) break;
            }
        }
        out.insert(N - 1);
    };
    upper_of(M.outgroup, M.upper);
    upper_of(M.conservedgroup, M.upper_conserve);
    return true;
}

struct ModelOut {
    double loglik = 0, max_loglik = 0;
    double rates[5] = {0, 0, 0, 0, 0};
    int failure = 0, n_configs = 0, done = 0;
    std::vector<int> max_z;
    std::vector<double> post_z;
    std::vector<double> tr_loglik, tr_n, tr_c, tr_g, tr_l, tr_l2;
    std::vector<int8_t> tr_z;
};

// ---------------------------------------------------------------------------
// BPP_C: one element (bpp_c.hpp:40-516, bpp_c.cpp, bpp_c2.cpp)
// ---------------------------------------------------------------------------
// One element's chain state carried from one SAMPLE_HYPER chain to the next:
// bpp.cur_Z[1][CC] and bpp.cur_{n,c,g,l,l2}rate[CC] (bpp.hpp:105,137-142),
// written at the end of Gibbs when UpHyper is set (bpp_c.cpp:475-485).  Z
// empty: the first chain's start (bpp_c.cpp:138-146).
struct CarryState {
    std::vector<int> Z;
    double n = 0, c = 0, g = 0, l = 0, l2 = 0;
};

struct Element {
    const Model& M;
    int S, N, GG = 0, CC = 0, root = 0;
    int num_burn, num_mcmc, adaptive_freq;
    std::vector<int> Tg;           // [GG][N]
    std::vector<double> lambda;    // [GG][N][4]
    std::vector<double> ambig;     // ambiguousS_null [GG][S][4]
    std::vector<int> c2a, c2b, parent2;
    std::vector<double> distances2;
    std::vector<int> nodes, internal_nodes, upper_c, upper_conserve_c;
    std::vector<char> missing;
    std::vector<Mat4> tm_null, tm_cons, tm_neut;
    std::vector<Mat3> log_TM_Int;
    double prior_z[3];
    std::vector<int> Z, fixZ, Max_Z;
    std::vector<std::vector<int>> trace_Z;
    std::vector<double> trace_loglik, trace_full_loglik, trace_n_rate, trace_c_rate, trace_l_rate, trace_l2_rate,
        trace_g_rate;
    std::vector<double> log_prob_back;  // [N][3]
    std::vector<double> log_emission;   // [N][3]
    double MaxLoglik = LOG_ZERO;
    int Max_m = 0, m = 0;
    int accept_n_rate = 0, accept_c_rate = 0;
    double prop_n = 0, prop_c = 0;
    bool failure = false;
    oracle_rng::Stream rng;

    double& lam(int g, int s, int k) { return lambda[((size_t)g * N + s) * 4 + k]; }
    double* lamv(int g, int s) { return &lambda[((size_t)g * N + s) * 4]; }
    int& tg(int g, int s) { return Tg[(size_t)g * N + s]; }

    explicit Element(const Model& m_) : M(m_) {}

    void getSubtree(int j, std::vector<int>& out) {  // bpp_c.cpp:44-60
        if (c2a[j] != -1) getSubtree(c2a[j], out);
        if (c2b[j] != -1) getSubtree(c2b[j], out);
        out.push_back(j);
    }

    void getSubtree_missing(int ss, const std::set<int>& up, int child) {  // bpp_c.cpp:64-113
        if (up.find(ss) == up.end() || ss < S) return;
        int s = ss;
        while (up.find(s) != up.end() && s >= S) {
            int p0 = c2a[s], p1 = c2b[s];
            if (missing[p0] && !missing[p1]) {
                parent2[p0] = -1;
                distances2[p1] += distances2[s];
                if (s == root) root = p1;
                else {
                    if (child == 0) c2a[parent2[ss]] = p1; else c2b[parent2[ss]] = p1;
                    parent2[p1] = parent2[ss];
                }
                s = p1;
            } else if (!missing[p0] && missing[p1]) {
                parent2[p1] = -1;
                distances2[p0] += distances2[s];
                if (s == root) root = p0;
                else {
                    if (child == 0) c2a[parent2[ss]] = p0; else c2b[parent2[ss]] = p0;
                    parent2[p0] = parent2[ss];
                }
                s = p0;
            } else {
                getSubtree_missing(p0, up, 0);
                getSubtree_missing(p1, up, 1);
                return;
            }
        }
    }

    // BPP_C ctor (bpp_c.hpp:143-476).  Returns true when the element is filtered.
    bool construct(int64_t cc, const uint8_t* bases, int len) {
        const pacc_opts& o = M.o;
        rng.set(o.seed);
        num_burn = o.burnin;
        num_mcmc = o.mcmc;
        adaptive_freq = o.adapt_freq;
        N = M.N;
        S = M.S;
        CC = (int)cc;
        GG = len;
        if (GG < o.min_len) return true;
        Tg.assign((size_t)GG * N, -1);
        root = N - 1;
        lambda.assign((size_t)GG * N * 4, 0.0);
        prior_z[0] = std::log(0.5); prior_z[1] = std::log(0.5); prior_z[2] = std::log(0.0);
        std::vector<int> num_missing(S, 0);
        const char gapchar = (char)o.gapchar;
        for (int s = 0; s < S; s++) {
            const uint8_t* y = bases + (size_t)s * len;
            for (int g = 0; g < GG; g++) {
                double* L = lamv(g, s);
                for (int k = 0; k < K; k++) L[k] = LOG_ZERO;
                switch ((char)y[g]) {
                    case 'a': L[0] = 0; tg(g, s) = 0; break;
                    case 'c': L[1] = 0; tg(g, s) = 1; break;
                    case 'g': L[2] = 0; tg(g, s) = 2; break;
                    case 't': L[3] = 0; tg(g, s) = 3; break;
                    case 'r': L[0] = 0; L[2] = 0; break;
                    case 'y': L[1] = 0; L[3] = 0; break;
                    case 'k': L[2] = 0; L[3] = 0; break;
                    case 'm': L[0] = 0; L[1] = 0; break;
                    case 's': L[1] = 0; L[2] = 0; break;
                    case 'w': L[0] = 0; L[3] = 0; break;
                    default:
                        for (int b = 0; b < K; b++) L[b] = 0;
                        if ((char)y[g] == gapchar) { tg(g, s) = 4; break; }
                        tg(g, s) = 5;
                }
            }
        }
        // column trimming (bpp_c.hpp:267-301)
        if (o.trim_gap_percent < 1) {
            std::vector<int> keep;
            int nmis_cols = 0;
            for (int g = 0; g < GG; g++) {
                int mis = 0;
                for (int s = 0; s < S; s++) if (tg(g, s) >= 4) mis++;
                if (mis > S * o.trim_gap_percent) nmis_cols++;
                else keep.push_back(g);
            }
            if (GG - nmis_cols < o.min_len) return true;
            std::vector<int> Tg2((size_t)keep.size() * N);
            std::vector<double> L2((size_t)keep.size() * N * 4);
            for (size_t i = 0; i < keep.size(); i++) {
                std::memcpy(&Tg2[i * N], &Tg[(size_t)keep[i] * N], sizeof(int) * N);
                std::memcpy(&L2[i * N * 4], &lambda[(size_t)keep[i] * N * 4], sizeof(double) * N * 4);
            }
            Tg.swap(Tg2);
            lambda.swap(L2);
            GG = (int)keep.size();
        }
        for (int s = 0; s < S; s++)
            for (int g = 0; g < GG; g++) if (tg(g, s) == 4) num_missing[s]++;
        ambig.assign((size_t)GG * S * 4, 0.0);
        c2a = M.ch0; c2b = M.ch1; parent2 = M.parent; distances2 = M.distances;
        // missing flags (bpp_c.hpp:331-351)
        missing.assign(N, 0);
        for (int s = S; s < N; s++) {
            int p[2] = {c2a[s], c2b[s]};
            for (int cc2 = 0; cc2 < 2; cc2++) {
                int chi = p[cc2];
                if (chi < S && num_missing[chi] > o.gap_prop * GG) missing[chi] = 1;
            }
            if (missing[p[0]] && missing[p[1]]) missing[s] = 1;
        }
        // conserved-species filter (bpp_c.hpp:361-373)
        int ct = 0;
        for (int c : M.conservedgroup) if (c >= 0 && c < N && missing[c]) ct++;
        if (ct > o.conserve_prop * (double)M.conservedgroup.size()) return true;
        // pruning (bpp_c.hpp:379-390)
        if (o.prune_tree) {
            std::set<int> alls;
            for (int s = 0; s < N; s++) alls.insert(s);
            getSubtree_missing(N - 1, alls, -1);
        } else {
            getSubtree_missing(N - 1, M.upper, -1);
        }
        parent2[root] = N;
        getSubtree(root, nodes);
        for (int s : nodes) {
            if (s >= S) internal_nodes.push_back(s);
            if (M.upper.count(s)) upper_c.push_back(s);
            if (M.upper_conserve.count(s)) upper_conserve_c.push_back(s);
        }
        // both children missing at a column -> K (bpp_c.hpp:417-428)
        for (int s : internal_nodes)
            for (int g = 0; g < GG; g++)
                if (tg(g, c2a[s]) >= K && tg(g, c2b[s]) >= K) tg(g, s) = K;
        size_t T = (size_t)num_burn + num_mcmc;
        trace_loglik.assign(T, 0); trace_full_loglik.assign(T, 0);
        trace_Z.assign(T, std::vector<int>(N, 1));
        trace_n_rate.assign(T, 0); trace_c_rate.assign(T, 0);
        trace_l_rate.assign(T, 0); trace_g_rate.assign(T, 0); trace_l2_rate.assign(T, 0);
        log_emission.assign((size_t)N * 3, 0.0);
        for (int s = 0; s < N; s++)
            if (missing[s]) {
                log_emission[s * 3 + 2] = std::log(1.0);   // nconsToMis = 1
                log_emission[s * 3 + 1] = std::log(o.cons_to_mis);
                log_emission[s * 3 + 0] = std::log(1.0);
            }
        tm_null.assign(N, Mat4{}); tm_cons.assign(N, Mat4{}); tm_neut.assign(N, Mat4{});
        for (int s = 0; s < N; s++)
            for (int a = 0; a < 4; a++)
                for (int b = 0; b < 4; b++) { tm_null[s].a[a][b] = 0; tm_cons[s].a[a][b] = 0; tm_neut[s].a[a][b] = 0; }
        log_TM_Int.assign(N, Mat3{});
        for (int s = 0; s < N; s++)
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) log_TM_Int[s].a[a][b] = 0;
        return false;
    }

    void getEmission_ambig() {  // bpp_c.cpp:116-128
        for (int s = 0; s < S; s++) {
            if (missing[s]) continue;
            for (int g = 0; g < GG; g++) {
                if (tg(g, s) != -1) continue;
                Vec4 y;
                for (int k = 0; k < K; k++) y.v[k] = lam(g, s, k);
                Vec4 r = log_multi(tm_null[s], y);
                for (int k = 0; k < K; k++) ambig[((size_t)g * S + s) * 4 + k] = r.v[k];
            }
        }
    }

    // initMCMC (bpp_c.cpp:131-343).  chain == 0: Z = 1 on the tree's nodes,
    // 0 at the root, -1 elsewhere (bpp_c.cpp:138-146).  A later chain takes
    // bpp.cur_Z[resZ][CC] (bpp_c.cpp:150), which only SAMPLE_HYPER updates
    // (bpp_c.cpp:475-477): without it that is the zero vector of bpp.cpp:201,
    // so the chain starts from Z = 0 on every node.  Everything else (rates,
    // proposal scales, the draw stream from SEED) starts as in chain 0.
    // carry: SAMPLE_HYPER's state (bpp_c.cpp:150,165-177): its Z, when set,
    // and its rates replace the start values.
    void initMCMC(int resZ, int chain = 0, const CarryState* carry = nullptr) {
        const pacc_opts& o = M.o;
        failure = false;
        prop_c = 1.2;
        prop_n = (double)1 / GG * 10;
        if (carry && !carry->Z.empty()) {
            Z = carry->Z;
        } else if (chain == 0) {
            Z.assign(N, -1);
            for (int s : nodes) Z[s] = 1;
            Z[root] = 0;
        } else {
            Z.assign(N, 0);
        }
        fixZ.assign(N, -1);
        for (int s : upper_c) fixZ[s] = 1;
        fixZ[root] = 1;
        MaxLoglik = LOG_ZERO;
        double init_lrate2 = (o.hyper_lrate2_a == 0) ? 0.0 : o.init_lrate2;  // main.cpp:286
        trace_n_rate[0] = carry ? carry->n : o.init_acce_rate;
        trace_c_rate[0] = carry ? carry->c : o.init_conserve_rate;
        trace_l_rate[0] = carry ? carry->l : o.init_lrate;
        trace_l2_rate[0] = carry ? carry->l2 : init_lrate2;
        trace_g_rate[0] = carry ? carry->g : o.init_grate;
        for (int s = 0; s < N; s++) tm_null[s] = M.log_cache_TM_null[s];
        for (size_t i = 0; i + 1 < nodes.size(); i++) {
            int s = nodes[i];
            if (distances2[s] > 1e-10) {
                if (distances2[s] != M.distances[s]) tm_null[s] = log_tm(M, distances2[s], 1.0, false);
                tm_neut[s] = log_tm(M, distances2[s], trace_n_rate[0], true);
                tm_cons[s] = log_tm(M, distances2[s], trace_c_rate[0], true);
            } else {
                tm_cons[s] = tm_null[s];
                tm_neut[s] = tm_null[s];
            }
        }
        log_prob_back.assign((size_t)N * 3, 0.0);
        for (int s = S; s < N; s++)
            for (int g = 0; g < GG; g++)
                for (int k = 0; k < K; k++) lam(g, s, k) = 0;
        getEmission_ambig();
        if (resZ == 2) {
            for (int s : upper_conserve_c) fixZ[s] = 1;
        } else if (resZ == 0) {
            for (size_t i = 0; i + 1 < nodes.size(); i++) fixZ[nodes[i]] = 1;
        }
        for (int s : nodes) {
            Mat3& t = log_TM_Int[s];
            if (fixZ[s] == 1) {
                t.a[0][1] = LOG_ZERO; t.a[1][1] = 0; t.a[2][1] = LOG_ZERO;
                t.a[0][0] = std::log(1 - trace_g_rate[0]); t.a[1][0] = std::log(trace_g_rate[0]); t.a[2][0] = LOG_ZERO;
            } else {
                t.a[0][0] = std::log(1 - trace_g_rate[0]); t.a[1][0] = std::log(trace_g_rate[0]); t.a[2][0] = LOG_ZERO;
                double y = 1 - trace_l_rate[0];
                t.a[0][1] = LOG_ZERO; t.a[1][1] = std::log(y); t.a[2][1] = std::log(1 - y);
                t.a[0][2] = LOG_ZERO; t.a[1][2] = std::log(trace_l2_rate[0]); t.a[2][2] = std::log(1 - trace_l2_rate[0]);
            }
        }
    }

    const Mat4& cache_for(int chi) const {
        if (Z[chi] == 2) return tm_neut[chi];
        if (Z[chi] == 0) return tm_null[chi];
        return tm_cons[chi];
    }

    // Update_Tg (bpp_c.cpp:644-739)
    void Update_Tg(int g, const std::vector<char>& visited, bool tosample) {
        if (!tosample) {
            for (int s : internal_nodes) {
                if (visited[s] || missing[s] || tg(g, s) >= K) continue;
                int p[2] = {c2a[s], c2b[s]};
                for (int cc = 0; cc < 2; cc++) {
                    int chi = p[cc];
                    if (missing[chi] || tg(g, chi) >= K) continue;
                    Vec4 y;
                    for (int k = 0; k < K; k++) y.v[k] = lam(g, chi, k);
                    Vec4 r = log_multi(cache_for(chi), y);
                    for (int k = 0; k < K; k++) lam(g, s, k) += r.v[k];
                }
            }
            if (!visited[root])
                for (int k = 0; k < K; k++) lam(g, root, k) += M.log_pi[k];
        } else {
            double prob[4];
            log_sample(lamv(g, root), K, prob);
            int nn = rng.categorical(K, prob);
            if (nn > K - 1 || nn < 0) throw std::runtime_error("Sample Tg root error");
            tg(g, root) = nn;
            for (int i = (int)internal_nodes.size() - 2; i >= 0; i--) {
                int s = internal_nodes[i];
                int p = parent2[s];
                if (missing[s] || tg(g, s) >= K) continue;
                const Mat4& T = cache_for(s);
                double lt[4], tp[4];
                int tp_col = tg(g, p);
                for (int k = 0; k < K; k++) lt[k] = T.a[k][tp_col] + lam(g, s, k);
                log_sample(lt, K, tp);
                int n2 = rng.categorical(K, tp);
                if (n2 > K - 1 || n2 < 0) throw std::runtime_error("Sample Tg error");
                tg(g, s) = n2;
            }
        }
    }

    // MonitorChain (bpp_c.cpp:741-834)
    void MonitorChain(double& loglik, double add_loglik, int resZ) {
        for (int s = 0; s < N; s++) trace_Z[m][s] = Z[s];
        if (m == 0) {
            trace_loglik[m] = 0;
            for (int g = 0; g < GG; g++) trace_loglik[m] += log_exp_sum(lamv(g, root), K);
            loglik = trace_loglik[m];
        } else {
            trace_loglik[m] = loglik;
        }
        trace_full_loglik[m] = trace_loglik[m] + add_loglik;
        trace_full_loglik[m] += log_gamma_pdf(trace_c_rate[m], M.o.conserve_prior_a, M.o.conserve_prior_b);
        if (resZ != 0) trace_full_loglik[m] += log_gamma_pdf(trace_n_rate[m], M.o.acce_prior_a, M.o.acce_prior_b);
        if (m >= num_burn && trace_full_loglik[m] > MaxLoglik) {
            MaxLoglik = trace_full_loglik[m];
            Max_Z = Z;
            Max_m = m;
        }
    }

    // getUpdateNode(changedZ) (bpp_c.cpp:620-642)
    void getUpdateNode(const std::vector<int>& changedZ, std::vector<char>& visited) {
        for (int i = 0; i < N; i++) visited[i] = 1;
        for (int i = (int)changedZ.size() - 1; i >= 0; i--) {
            int j = parent2[changedZ[i]];
            while (j != N) {
                if (!visited[j]) break;
                visited[j] = 0;
                for (int g = 0; g < GG; g++)
                    for (int k = 0; k < K; k++) lam(g, j, k) = 0;
                j = parent2[j];
            }
        }
    }

    // getUpdateNode(neut) (bpp_c.cpp:836-858)
    void getUpdateNode(bool neut, std::vector<char>& visited) {
        for (int s : nodes) {
            if (missing[s]) continue;
            if (!neut && (Z[s] == 0 || Z[s] == 2)) continue;
            if (neut && (Z[s] == 1 || Z[s] == 0)) continue;
            int j = parent2[s];
            while (j != N) {
                if (!visited[j]) break;
                visited[j] = 0;
                j = parent2[j];
            }
        }
    }

    // log_f_Xz (bpp_c.cpp:860-928)
    double log_f_Xz(const std::vector<char>& visited, std::vector<double>& lt, bool neut, double propos) {
        auto L = [&](int g, int s) { return &lt[((size_t)g * N + s) * 4]; };
        for (int s : internal_nodes) {
            if (visited[s]) continue;
            int p[2] = {c2a[s], c2b[s]};
            for (int cc = 0; cc < 2; cc++) {
                int chi = p[cc];
                if (missing[chi]) continue;
                Mat4 transition;
                if (!neut) {
                    if (Z[chi] == 1) transition = log_tm(M, distances2[chi], propos, true);
                    else if (Z[chi] == 2) transition = tm_neut[chi];
                    else transition = tm_null[chi];
                } else {
                    if (Z[chi] == 2) transition = log_tm(M, distances2[chi], propos, true);
                    else if (Z[chi] == 1) transition = tm_cons[chi];
                    else transition = tm_null[chi];
                }
                for (int g = 0; g < GG; g++) {
                    if (tg(g, chi) < K) {
                        Vec4 y;
                        double* c = L(g, chi);
                        for (int k = 0; k < K; k++) y.v[k] = c[k];
                        Vec4 r = log_multi(transition, y);
                        double* d = L(g, s);
                        for (int k = 0; k < K; k++) d[k] += r.v[k];
                    }
                }
            }
        }
        double result = 0;
        for (int g = 0; g < GG; g++) {
            double* d = L(g, root);
            if (!visited[root])
                for (int k = 0; k < K; k++) d[k] += M.log_pi[k];
            result += log_exp_sum(d, K);
        }
        return result;
    }

    // sample_rate (bpp_c.cpp:930-1176), M = 1, adaptive, factor 0.5
    double sample_rate(int resZ, double old_rate, bool neut, const std::vector<char>& visited, double& loglik_old) {
        const pacc_opts& o = M.o;
        const double adaptive_factor = 0.5;
        double cur_r = old_rate, prior_a, prior_b;
        if (neut) { prior_a = o.acce_prior_a; prior_b = o.acce_prior_b; }
        else { prior_a = o.conserve_prior_a; prior_b = o.conserve_prior_b; }
        if (visited[root]) {
            if (resZ != 0) {
                cur_r = rng.gamma(prior_a, prior_b);
                if (neut) {
                    if (o.ropt == 1 && cur_r < o.nlb) cur_r = old_rate;
                    else if (o.ropt == 2 && cur_r < trace_c_rate[m]) cur_r = old_rate;
                } else {
                    if (o.ropt == 1 && cur_r > o.cub) cur_r = old_rate;
                    else if (o.ropt == 2 && cur_r > trace_n_rate[m + 1]) cur_r = old_rate;
                }
            } else {
                cur_r = old_rate;
            }
        } else {
            std::vector<double> lt((size_t)GG * N * 4, 0.0);
            for (size_t i = 0; i + 1 < nodes.size(); i++) {
                int s = nodes[i];
                if (!visited[s]) continue;
                for (int g = 0; g < GG; g++)
                    for (int k = 0; k < K; k++) lt[((size_t)g * N + s) * 4 + k] = lam(g, s, k);
            }
            do {
                double r = rng.uniform();
                double proposal;
                if (neut) {
                    proposal = rng.gamma(cur_r / prop_n, prop_n);
                    if (o.ropt == 1 && proposal < o.nlb) break;
                    else if (o.ropt == 2 && proposal < trace_c_rate[m]) break;
                } else {
                    double u = r * (prop_c - 1 / prop_c) + 1 / prop_c;
                    proposal = cur_r * u;
                    if (o.ropt == 1 && proposal > o.cub) break;
                    else if (o.ropt == 2 && proposal > trace_n_rate[m + 1]) break;
                }
                if (proposal < 1e-12 || proposal > 1e8) break;
                double loglik_new = log_f_Xz(visited, lt, neut, proposal);
                double MH;
                if (neut)
                    MH = loglik_new - loglik_old + log_gamma_pdf(proposal, prior_a, prior_b) -
                         log_gamma_pdf(cur_r, prior_a, prior_b) + log_gamma_pdf(cur_r, proposal / prop_n, prop_n) -
                         log_gamma_pdf(proposal, cur_r / prop_n, prop_n);
                else
                    MH = loglik_new - loglik_old + log_gamma_pdf(proposal, prior_a, prior_b) -
                         log_gamma_pdf(cur_r, prior_a, prior_b) + std::log(cur_r) - std::log(proposal);
                if (std::log(r) < MH) {
                    cur_r = proposal;
                    loglik_old = loglik_new;
                    for (int s : internal_nodes) {
                        if (visited[s]) continue;
                        for (int g = 0; g < GG; g++)
                            for (int k = 0; k < K; k++) lam(g, s, k) = lt[((size_t)g * N + s) * 4 + k];
                    }
                }
            } while (false);
        }
        if (old_rate != cur_r) {
            for (size_t i = 0; i + 1 < nodes.size(); i++) {
                int s = nodes[i];
                if (distances2[s] < 1e-10) continue;
                if (neut) tm_neut[s] = log_tm(M, distances2[s], cur_r, true);
                else tm_cons[s] = log_tm(M, distances2[s], cur_r, true);
            }
            if (neut) accept_n_rate += 1; else accept_c_rate += 1;
        }
        if ((m + 1) % adaptive_freq == 0) {
            double scale_adj;
            int blocks = (m + 1) / adaptive_freq;
            double step = std::min(adaptive_factor, 1 / std::sqrt((double)blocks));
            if (neut) {
                double rate = (double)accept_n_rate / adaptive_freq;
                if (rate > 0.44) scale_adj = std::exp(step);
                else if (rate < 0.23) scale_adj = std::exp(-step);
                else scale_adj = 1;
                prop_n = prop_n * scale_adj;
                if (prop_n > 1) prop_n = 1;
                accept_n_rate = 0;
            } else {
                double rate = (double)accept_c_rate / adaptive_freq;
                if (rate > 0.44) scale_adj = std::exp(step);
                else if (rate < 0.23) scale_adj = std::exp(-step);
                else scale_adj = 1;
                prop_c = std::pow(prop_c, scale_adj);
                if (prop_c < 1.0001) prop_c = 1.0001;
                accept_c_rate = 0;
            }
        }
        return cur_r;
    }

    // getEmission (bpp_c2.cpp:355-390)
    void getEmission() {
        for (size_t i = 0; i + 1 < nodes.size(); i++) {
            int s = nodes[i];
            int p = parent2[s];
            if (missing[s]) continue;
            double e0 = 0, e1 = 0, e2 = 0;
            for (int g = 0; g < GG; g++) {
                int ts = tg(g, s);
                if (ts >= K) continue;
                int tp = tg(g, p);
                if (ts == -1) {
                    e0 += ambig[((size_t)g * S + s) * 4 + tp];
                    double v1[4], v2[4];
                    for (int k = 0; k < K; k++) {
                        v1[k] = tm_cons[s].a[k][tp] + lam(g, s, k);
                        v2[k] = tm_neut[s].a[k][tp] + lam(g, s, k);
                    }
                    e1 += log_exp_sum(v1, K);
                    e2 += log_exp_sum(v2, K);
                } else {
                    e0 += tm_null[s].a[ts][tp];
                    e1 += tm_cons[s].a[ts][tp];
                    e2 += tm_neut[s].a[ts][tp];
                }
            }
            log_emission[s * 3 + 0] = e0;
            log_emission[s * 3 + 1] = e1;
            log_emission[s * 3 + 2] = e2;
        }
    }

    // BPP::log_multi2 (bpp.hpp:447-460)
    void log_multi2(const Mat3& lx, const double* ly, double* out) {
        for (int i = 0; i < 3; i++) {
            double t[3];
            double mx = 0;
            for (int r = 0; r < 3; r++) {
                t[r] = lx.a[r][i] + ly[r];
                if (r == 0 || t[r] > mx) mx = t[r];
            }
            double s = 0;
            for (int r = 0; r < 3; r++) s += std::exp(t[r] - mx);
            out[i] = std::log(s) + mx;
        }
    }

    // Update_Z_subtree (bpp_c.cpp:1182-1293)
    std::vector<int> Update_Z_subtree() {
        getEmission();
        for (int s : nodes) {
            for (int k = 0; k < 3; k++) log_prob_back[s * 3 + k] = log_emission[s * 3 + k];
            if (fixZ[s] == 1) log_prob_back[s * 3 + 2] = LOG_ZERO;
        }
        for (size_t i = 0; i + 1 < nodes.size(); i++) {
            int s = nodes[i];
            int p = parent2[s];
            double msg[3];
            log_multi2(log_TM_Int[s], &log_prob_back[s * 3], msg);
            for (int k = 0; k < 3; k++) log_prob_back[p * 3 + k] += msg[k];
        }
        std::vector<int> changedZ;
        for (int k = 0; k < 3; k++) log_prob_back[root * 3 + k] += prior_z[k];
        double prob[3];
        log_sample(&log_prob_back[root * 3], 3, prob);
        int nn = rng.categorical(3, prob);
        int old = Z[root];
        Z[root] = nn;
        if (old != nn) changedZ.push_back(root);
        for (int i = (int)nodes.size() - 2; i >= 0; i--) {
            int s = nodes[i];
            int p = parent2[s];
            old = Z[s];
            double lt[3], tp[3];
            int zp = Z[p];
            for (int k = 0; k < 3; k++) lt[k] = log_TM_Int[s].a[k][zp] + log_prob_back[s * 3 + k];
            log_sample(lt, 3, tp);
            int n2 = rng.categorical(3, tp);
            Z[s] = n2;
            if (old != Z[s]) changedZ.push_back(s);
        }
        return changedZ;
    }

    // sample_transition (bpp_c.cpp:522-613)
    void sample_transition(double& gr, double& lr, double& lr2) {
        const pacc_opts& o = M.o;
        double nZ[3][3] = {{0}};
        for (size_t i = 0; i + 1 < nodes.size(); i++) {
            int p = parent2[nodes[i]];
            nZ[Z[nodes[i]]][Z[p]] += 1;
        }
        gr = rng.beta(o.hyper_grate_a + nZ[1][0] + nZ[2][0], o.hyper_grate_b + nZ[0][0]);
        for (size_t i = 0; i + 1 < nodes.size(); i++) {
            if (fixZ[nodes[i]] == 1) {
                int p = parent2[nodes[i]];
                nZ[Z[nodes[i]]][Z[p]] -= 1;
            }
        }
        lr = rng.beta(o.hyper_lrate_a + nZ[2][1], o.hyper_lrate_b + nZ[1][1]);
        if (o.hyper_lrate2_a == 0) lr2 = 0;
        else lr2 = rng.beta(o.hyper_lrate2_a + nZ[1][2], o.hyper_lrate2_b + nZ[2][2]);
        for (int s : nodes) {
            Mat3& t = log_TM_Int[s];
            if (fixZ[s] == 1) {
                t.a[1][1] = 0; t.a[2][1] = LOG_ZERO;
                t.a[0][0] = std::log(1 - gr); t.a[1][0] = std::log(gr); t.a[2][0] = LOG_ZERO;
            } else {
                t.a[0][0] = std::log(1 - gr); t.a[1][0] = std::log(gr); t.a[2][0] = LOG_ZERO;
                double y = 1 - lr;
                t.a[1][1] = std::log(y); t.a[2][1] = std::log(1 - y);
                t.a[1][2] = std::log(lr2); t.a[2][2] = std::log(1 - lr2);
            }
        }
    }

    // Gibbs (bpp_c.cpp:346-519) with UpR = true, UpHyper = false
    void Gibbs(int resZ, double& max_loglik_out, std::vector<int>& max_z_out) {
        std::vector<int> changedZ;
        std::vector<char> visited(N, 0);
        double logp_Z = 0.0;
        for (int g = 0; g < GG; g++) Update_Tg(g, visited, false);
        double log_lik_old = 0;
        for (m = 0; m < num_burn + num_mcmc; m++) {
            MonitorChain(log_lik_old, logp_Z, resZ);
            if (failure || (m == num_burn + num_mcmc - 1)) break;
            for (int g = 0; g < GG; g++) Update_Tg(g, visited, true);
            changedZ = Update_Z_subtree();
            getUpdateNode(changedZ, visited);
            if (!changedZ.empty()) {
                log_lik_old = 0;
                for (int g = 0; g < GG; g++) {
                    Update_Tg(g, visited, false);
                    log_lik_old += log_exp_sum(lamv(g, root), K);
                }
            }
            std::vector<char> vn(N, 1), vc(N, 1);
            getUpdateNode(true, vn);
            getUpdateNode(false, vc);
            trace_n_rate[m + 1] = sample_rate(resZ, trace_n_rate[m], true, vn, log_lik_old);
            trace_c_rate[m + 1] = sample_rate(resZ, trace_c_rate[m], false, vc, log_lik_old);
            sample_transition(trace_g_rate[m + 1], trace_l_rate[m + 1], trace_l2_rate[m + 1]);
        }
        max_loglik_out = MaxLoglik;
        max_z_out = Max_Z;
    }

    // Eval2 (bpp_c2.cpp:14-353).  Returns VB and the number of configurations.
    double Eval2(int resZ, int& n_conf_out, bool& fail) {
        const pacc_opts& o = M.o;
        Z = Max_Z;
        std::vector<int> posterior_Z(N, 0);
        std::vector<int> uncertainZ;
        for (int s = 0; s < N; s++) {
            for (size_t i = num_burn; i < trace_Z.size(); i++)
                if (trace_Z[i][s] == Max_Z[s]) posterior_Z[s]++;
            if (posterior_Z[s] < num_mcmc) uncertainZ.push_back(s);
        }
        std::vector<std::vector<int>> configZ;
        std::vector<int> numConfigZ;
        configZ.push_back(Max_Z);
        numConfigZ.push_back(0);
        unsigned numConf = 1;
        std::vector<double> var_nrate(1, 0), mean_nrate(1, 0), var_crate(1, 0), mean_crate(1, 0), cov_rate(1, 0),
            sum_full_loglik(1, 0);
        for (int i = (int)trace_Z.size() - 1; i >= num_burn; i--) {
            unsigned j = 0;
            for (; j < numConf; j++) {
                size_t u = 0;
                for (; u < uncertainZ.size(); u++)
                    if (trace_Z[i][uncertainZ[u]] != configZ[j][uncertainZ[u]]) break;
                if (u == uncertainZ.size()) break;
            }
            if (j == numConf) {
                configZ.push_back(trace_Z[i]);
                numConf++;
                numConfigZ.push_back(0);
                var_crate.push_back(0); var_nrate.push_back(0);
                mean_crate.push_back(0); mean_nrate.push_back(0);
                cov_rate.push_back(0); sum_full_loglik.push_back(0);
            }
            numConfigZ[j]++;
            var_crate[j] += std::pow(trace_c_rate[i], 2);
            mean_crate[j] += trace_c_rate[i];
            if (resZ != 0) {
                var_nrate[j] += std::pow(trace_n_rate[i], 2);
                mean_nrate[j] += trace_n_rate[i];
                cov_rate[j] += trace_c_rate[i] * trace_n_rate[i];
            }
            sum_full_loglik[j] += trace_full_loglik[i] / num_mcmc;
        }
        double VB = 0, logdet = 0;
        int effective_sum = 0;
        auto priorZ_of = [&](const std::vector<int>& cz) {
            double nZ[3][3] = {{0}};
            for (size_t k = 0; k + 1 < nodes.size(); k++) nZ[cz[nodes[k]]][cz[parent2[nodes[k]]]] += 1;
            double pz = lnbeta(o.hyper_grate_a + nZ[1][0] + nZ[2][0], o.hyper_grate_b + nZ[0][0]) -
                        lnbeta(o.hyper_grate_a, o.hyper_grate_b);
            for (size_t k = 0; k + 1 < nodes.size(); k++)
                if (fixZ[nodes[k]] == 1) nZ[cz[nodes[k]]][cz[parent2[nodes[k]]]] -= 1;
            pz += lnbeta(o.hyper_lrate_a + nZ[2][1], o.hyper_lrate_b + nZ[1][1]) -
                  lnbeta(o.hyper_lrate_a, o.hyper_lrate_b);
            if (o.hyper_lrate2_a > 0)
                pz += lnbeta(o.hyper_lrate2_a + nZ[1][2], o.hyper_lrate2_b + nZ[2][2]) -
                      lnbeta(o.hyper_lrate2_a, o.hyper_lrate2_b);
            pz += prior_z[cz[root]];
            return pz;
        };
        for (unsigned i = 0; i < numConf; i++) {
            double w = (double)numConfigZ[i] / num_mcmc;
            if (w < 0.02) continue;
            double priorZ = priorZ_of(configZ[i]);
            sum_full_loglik[i] += numConfigZ[i] * priorZ / num_mcmc;
            if (resZ == 0) {
                logdet = std::log(var_crate[i] - std::pow(mean_crate[i], 2) / numConfigZ[i]) - std::log(numConfigZ[i]);
            } else {
                double vc = var_crate[i] - std::pow(mean_crate[i], 2) / numConfigZ[i];
                double vn = var_nrate[i] - std::pow(mean_nrate[i], 2) / numConfigZ[i];
                double cov = cov_rate[i] - mean_nrate[i] * mean_crate[i] / numConfigZ[i];
                logdet = std::log(vc * vn - cov * cov) - 2 * std::log(numConfigZ[i]);
            }
            if (std::isnan(logdet)) continue;
            effective_sum += numConfigZ[i];
            VB -= w * std::log(numConfigZ[i]);
            VB += sum_full_loglik[i];
            VB += 0.5 * logdet * numConfigZ[i] / num_mcmc;
        }
        if (effective_sum == 0) {
            double varn = 0, varc = 0, cov = 0, meann = 0, meanc = 0;
            VB = 0;
            for (unsigned i = 0; i < numConf; i++) {
                varc += var_crate[i];
                meanc += mean_crate[i];
                if (resZ != 0) { meann += mean_nrate[i]; varn += var_nrate[i]; cov += cov_rate[i]; }
            }
            double rn = meann / num_mcmc;
            double rc = meanc / num_mcmc;
            for (size_t k = 0; k + 1 < nodes.size(); k++) {
                int s = nodes[k];
                tm_cons[s] = log_tm(M, distances2[s], rc, true);
                if (resZ != 0) tm_neut[s] = log_tm(M, distances2[s], rn, true);
            }
            std::vector<char> visited(N, 0);
            for (unsigned i = 0; i < numConf; i++) {
                double priorZ = priorZ_of(configZ[i]);
                Z = configZ[i];
                for (int s = S; s < N; s++)
                    for (int g = 0; g < GG; g++)
                        for (int k = 0; k < K; k++) lam(g, s, k) = 0;
                sum_full_loglik[i] = 0;
                for (int g = 0; g < GG; g++) {
                    Update_Tg(g, visited, false);
                    sum_full_loglik[i] += log_exp_sum(lamv(g, root), K);
                }
                sum_full_loglik[i] += priorZ;
            }
            VB = log_exp_sum(sum_full_loglik.data(), (int)sum_full_loglik.size());
            VB += log_gamma_pdf(rc, o.conserve_prior_a, o.conserve_prior_b);
            if (resZ != 0) VB += log_gamma_pdf(rn, o.acce_prior_a, o.acce_prior_b);
            if (resZ == 0) {
                varc -= std::pow(meanc, 2) / num_mcmc;
                logdet = std::log(varc) - std::log(num_mcmc);
                VB += 0.5 * logdet + 0.5 * std::log(2 * M_PI);
            } else {
                varn -= std::pow(meann, 2) / num_mcmc;
                varc -= std::pow(meanc, 2) / num_mcmc;
                cov -= meann * meanc / num_mcmc;
                logdet = std::log(varc * varn - cov * cov) - 2 * std::log(num_mcmc);
                VB += 0.5 * logdet + std::log(2 * M_PI);
            }
        } else {
            if (resZ != 0) VB = VB * ((double)num_mcmc / effective_sum) + std::log(num_mcmc) + std::log(2 * M_PI) + 1;
            else VB = VB * ((double)num_mcmc / effective_sum) + std::log(num_mcmc) + 0.5 * (std::log(2 * M_PI) + 1);
        }
        n_conf_out = (int)numConf;
        fail = std::isnan(VB);
        return VB;
    }

    // Output_init (bpp_c2.cpp:739-785)
    void Output_init(ModelOut& out) {
        auto median = [](std::vector<double>& v) {
            std::sort(v.begin(), v.end());
            return v[v.size() / 2];
        };
        out.rates[0] = median(trace_n_rate);
        out.rates[1] = median(trace_c_rate);
        out.rates[2] = median(trace_g_rate);
        out.rates[3] = median(trace_l_rate);
        out.rates[4] = median(trace_l2_rate);
        out.post_z.assign((size_t)N * 4, 0.0);
        std::vector<int> countZ((size_t)N * 4, 0);
        for (int s = 0; s < N; s++) {
            for (size_t i = num_burn; i < trace_loglik.size(); i++) countZ[s * 4 + trace_Z[i][s] + 1]++;
            if (missing[s]) countZ[s * 4 + 0] = num_mcmc;
        }
        for (int s = 0; s < N; s++)
            for (int k = 0; k < 4; k++) out.post_z[s * 4 + k] = (double)countZ[s * 4 + k] / num_mcmc;
    }

    void record_trace(ModelOut& out, int T) {
        T = std::min<int>(T, (int)trace_loglik.size());
        out.tr_loglik.assign(trace_loglik.begin(), trace_loglik.begin() + T);
        out.tr_n.assign(trace_n_rate.begin(), trace_n_rate.begin() + T);
        out.tr_c.assign(trace_c_rate.begin(), trace_c_rate.begin() + T);
        out.tr_g.assign(trace_g_rate.begin(), trace_g_rate.begin() + T);
        out.tr_l.assign(trace_l_rate.begin(), trace_l_rate.begin() + T);
        out.tr_l2.assign(trace_l2_rate.begin(), trace_l2_rate.begin() + T);
        out.tr_z.assign((size_t)T * N, 0);
        for (int i = 0; i < T; i++)
            for (int s = 0; s < N; s++) out.tr_z[(size_t)i * N + s] = (int8_t)trace_Z[i][s];
    }
};

// carry set: a SAMPLE_HYPER chain — only the full model M2 runs
// (main.cpp:466-494), from the carried state, which it then updates.
void run_one(const Model& M, const pacc_element_batch* b, int e, pacc_result* res, int chain = 0,
             CarryState* carry = nullptr) {
    const pacc_opts& o = M.o;
    const int N = M.N;
    res->element_no = b->element_no ? b->element_no[e] : e;
    res->n_nodes = N;
    res->status = PACC_OK;
    for (int r = 0; r < 3; r++) std::memset(&res->model[r], 0, sizeof(pacc_model_result));
    if (res->max_z) std::memset(res->max_z, 0, sizeof(int32_t) * 3 * N);
    if (res->post_z) std::memset(res->post_z, 0, sizeof(double) * 3 * N * 4);
    Element E(M);
    bool filtered = E.construct(res->element_no, b->bases + b->offsets[e], b->lengths[e]);
    if (filtered) { res->status = PACC_FILTERED; return; }
    // main.cpp:468-494: M0 (resZ 0), M1 (resZ 2), M2 (resZ 1)
    const int resZ_of[3] = {0, 2, 1};
    try {
        for (int mi = carry ? 2 : 0; mi < 3; mi++) {
            int resZ = resZ_of[mi];
            ModelOut out;
            E.initMCMC(resZ, chain, carry);
            std::vector<int> maxz;
            double maxll;
            E.Gibbs(resZ, maxll, maxz);
            if (carry) {   // bpp_c.cpp:475-485: the state where Gibbs stopped
                carry->Z = E.Z;
                carry->n = E.trace_n_rate[E.m];
                carry->c = E.trace_c_rate[E.m];
                carry->g = E.trace_g_rate[E.m];
                carry->l = E.trace_l_rate[E.m];
                carry->l2 = E.trace_l2_rate[E.m];
                if (res->end_z)
                    for (int s = 0; s < N; s++) res->end_z[s] = (int8_t)carry->Z[s];
                const double v[5] = {carry->n, carry->c, carry->g, carry->l, carry->l2};
                for (int q = 0; q < 5; q++) res->end_rates[q] = v[q];
            }
            if (o.trace_iters > 0) E.record_trace(out, o.trace_iters);
            bool fail = false;
            int nconf = 0;
            double vb = E.Eval2(resZ, nconf, fail);
            E.Output_init(out);
            pacc_model_result& mr = res->model[mi];
            mr.loglik = vb;
            mr.max_loglik = maxll;
            mr.n_rate = out.rates[0]; mr.c_rate = out.rates[1]; mr.g_rate = out.rates[2];
            mr.l_rate = out.rates[3]; mr.l2_rate = out.rates[4];
            mr.failure = fail ? 1 : 0;
            mr.n_configs = nconf;
            if (fail) res->status = PACC_NAN_LIKELIHOOD;
            if (res->max_z)
                for (int s = 0; s < N; s++) res->max_z[mi * N + s] = (s < (int)maxz.size()) ? maxz[s] : 0;
            if (res->post_z)
                for (int i = 0; i < N * 4; i++) res->post_z[(size_t)mi * N * 4 + i] = out.post_z[i];
            int T = o.trace_iters;
            if (T > 0) {
                pacc_trace& tr = res->trace;
                int n = (int)out.tr_loglik.size();
                for (int i = 0; i < n; i++) {
                    if (tr.loglik) tr.loglik[mi * T + i] = out.tr_loglik[i];
                    if (tr.n_rate) tr.n_rate[mi * T + i] = out.tr_n[i];
                    if (tr.c_rate) tr.c_rate[mi * T + i] = out.tr_c[i];
                    if (tr.g_rate) tr.g_rate[mi * T + i] = out.tr_g[i];
                    if (tr.l_rate) tr.l_rate[mi * T + i] = out.tr_l[i];
                    if (tr.l2_rate) tr.l2_rate[mi * T + i] = out.tr_l2[i];
                    if (tr.z)
                        for (int s = 0; s < N; s++) tr.z[((size_t)mi * T + i) * N + s] = out.tr_z[(size_t)i * N + s];
                }
            }
        }
    } catch (std::exception&) {
        res->status = PACC_SAMPLER_ERROR;
    }
}

}  // namespace

extern "C" {

// Runs every element of the batch through M0, M1, M2 on the CPU, elements
// spread over n_threads OpenMP threads like main.cpp:452 (schedule guided).
int oracle_run(const pacc_model* model, const pacc_opts* opts, const pacc_element_batch* batch, pacc_result* out,
               int n_threads) {
    Model M;
    if (!build_model(model, opts, M)) return PACC_EINVAL;
    if (opts->indel != 0) return PACC_EUNSUPPORTED;
#ifdef _OPENMP
    if (n_threads <= 0) n_threads = omp_get_max_threads();
#pragma omp parallel for schedule(guided) num_threads(n_threads)
#endif
    for (int e = 0; e < batch->n_elements; e++) run_one(M, batch, e, &out[e]);
    return PACC_OK;
}

// The same for chain `chain` of a CHAIN > 1 run (main.cpp:445): each element
// runs again from SEED with the continued-chain start of initMCMC.
int oracle_run_chain(const pacc_model* model, const pacc_opts* opts, const pacc_element_batch* batch,
                     pacc_result* out, int n_threads, int chain) {
    Model M;
    if (!build_model(model, opts, M)) return PACC_EINVAL;
    if (opts->indel != 0) return PACC_EUNSUPPORTED;
    if (chain < 0) return PACC_EINVAL;
#ifdef _OPENMP
    if (n_threads <= 0) n_threads = omp_get_max_threads();
#pragma omp parallel for schedule(guided) num_threads(n_threads)
#endif
    for (int e = 0; e < batch->n_elements; e++) run_one(M, batch, e, &out[e], chain);
    return PACC_OK;
}

// SAMPLE_HYPER: CHAIN chains of M2 over the batch, each from the state the
// previous one left (main.cpp:445-509), with the hyper-parameters drawn
// between chains by BPP::sample_hyperparam (bpp.cpp:324-477) from the model's
// own generator (seeded with SEED, bpp.hpp:177-178).  out: [n_chains][n]
// results (model[2] filled); hyper: [n_chains + 1][10] = (nprior_a, nprior_b,
// cprior_a, cprior_b, prior_l_a, prior_l_b, prior_g_a, prior_g_b, prior_l2_a,
// prior_l2_b), row 0 the starting values and row k + 1 those after chain k.
int oracle_run_hyper(const pacc_model* model, const pacc_opts* opts, const pacc_element_batch* batch,
                     int n_chains, pacc_result* out, double* hyper, int n_threads) {
    Model M0;
    if (!build_model(model, opts, M0)) return PACC_EINVAL;
    if (opts->indel != 0) return PACC_EUNSUPPORTED;
    const int n = batch->n_elements;
    double h[10] = {opts->acce_prior_a, opts->acce_prior_b, opts->conserve_prior_a, opts->conserve_prior_b,
                    opts->hyper_lrate_a, opts->hyper_lrate_b, opts->hyper_grate_a, opts->hyper_grate_b,
                    opts->hyper_lrate2_a, opts->hyper_lrate2_b};
    for (int q = 0; q < 10; q++) hyper[q] = h[q];
    // bpp.cpp:215-220: every element starts from the INIT_* values
    std::vector<CarryState> st(n);
    for (auto& c : st) {
        c.n = opts->init_acce_rate;
        c.c = opts->init_conserve_rate;
        c.g = opts->init_grate;
        c.l = opts->init_lrate;
        c.l2 = (opts->hyper_lrate2_a == 0) ? 0.0 : opts->init_lrate2;   // main.cpp:286
    }
    oracle_rng::Stream rng;
    rng.set(opts->seed);
#ifdef _OPENMP
    if (n_threads <= 0) n_threads = omp_get_max_threads();
#endif
    for (int chain = 0; chain < n_chains; chain++) {
        pacc_opts oc = *opts;
        oc.acce_prior_a = h[0]; oc.acce_prior_b = h[1];
        oc.conserve_prior_a = h[2]; oc.conserve_prior_b = h[3];
        oc.hyper_lrate_a = h[4]; oc.hyper_lrate_b = h[5];
        oc.hyper_grate_a = h[6]; oc.hyper_grate_b = h[7];
        oc.hyper_lrate2_a = h[8]; oc.hyper_lrate2_b = h[9];
        Model M;
        if (!build_model(model, &oc, M)) return PACC_EINVAL;
        pacc_result* res = out + (size_t)chain * n;
#ifdef _OPENMP
#pragma omp parallel for schedule(guided) num_threads(n_threads)
#endif
        for (int e = 0; e < n; e++) run_one(M, batch, e, &res[e], chain, &st[e]);
        // sample_hyperparam (bpp.cpp:324-477): independent MH on each pair,
        // sums over the batch's elements in order (filtered ones included
        // with the values they started from)
        const double p = 1, r = 1, q = 0.1, s = 0.1;
        const double vna = 100, vnb = 100, vca = 100, vcb = 100;
        const double ne = (double)n;
        double nap = rng.gamma(vna, h[0] / vna);
        double cap = rng.gamma(vca, h[2] / vca);
        double nbp = rng.gamma(vnb, h[1] / vnb);
        double cbp = rng.gamma(vcb, h[3] / vcb);
        auto rate_ratio = [&](double ap, double bp, double a, double b, double sum_r, double lpr) {
            double mr = (ap - 1) * (std::log(p) + lpr) - (q + sum_r) / bp - (ne + r) * std::lgamma(ap) -
                        std::log(bp) * ap * (s + ne);
            mr -= (a - 1) * (std::log(p) + lpr) - (q + sum_r) / b - (ne + r) * std::lgamma(a) -
                  std::log(b) * a * (s + ne);
            return mr;
        };
        {
            double sum_r = 0, lpr = 0;
            for (int e = 0; e < n; e++) { sum_r += st[e].n; lpr += std::log(st[e].n); }
            double mr = rate_ratio(nap, nbp, h[0], h[1], sum_r, lpr);
            double hr = std::log(gamma_pdf(h[0], vna, nap / vna)) - std::log(gamma_pdf(nap, vna, h[0] / vna)) +
                        std::log(gamma_pdf(h[1], vnb, nbp / vnb)) - std::log(gamma_pdf(nbp, vnb, h[1] / vnb));
            if (std::log(rng.uniform()) < mr + hr) { h[0] = nap; h[1] = nbp; }
        }
        {
            double sum_r = 0, lpr = 0;
            for (int e = 0; e < n; e++) { sum_r += st[e].c; lpr += std::log(st[e].c); }
            double mr = rate_ratio(cap, cbp, h[2], h[3], sum_r, lpr);
            double hr = std::log(gamma_pdf(h[2], vca, cap / vca)) - std::log(gamma_pdf(cap, vca, h[2] / vca)) +
                        std::log(gamma_pdf(h[3], vcb, cbp / vcb)) - std::log(gamma_pdf(cbp, vcb, h[3] / vcb));
            if (std::log(rng.uniform()) < mr + hr) { h[2] = cap; h[3] = cbp; }
        }
        // Beta hyper-parameters of l, l2, g: multiplicative U(0.7, 1.3) proposals
        auto beta_pair = [&](double& a, double& b, double CarryState::*f) {
            double u = rng.uniform() * (1.3 - 0.7) + 0.7;
            double ap = a * u;
            u = rng.uniform() * (1.3 - 0.7) + 0.7;
            double bp = b * u;
            double log_p = 0, log_pc = 0;
            for (int e = 0; e < n; e++) { log_p += std::log(st[e].*f); log_pc += std::log(1 - st[e].*f); }
            double mr = (ap - a) * (log_p - 1) + (bp - b) * (log_pc - 1);
            mr += ne * (lnbeta(a, b) - lnbeta(ap, bp));
            double hr = std::log(a) - std::log(ap) + std::log(b) - std::log(bp);
            if (std::log(rng.uniform()) < mr + hr) { a = ap; b = bp; }
        };
        beta_pair(h[4], h[5], &CarryState::l);
        beta_pair(h[8], h[9], &CarryState::l2);
        beta_pair(h[6], h[7], &CarryState::g);
        for (int k = 0; k < 10; k++) hyper[(size_t)(chain + 1) * 10 + k] = h[k];
    }
    return PACC_OK;
}

// Column encoding of one element (bpp_c.hpp:204-264, 267-301, 331-428):
// Tg codes after trimming [n_cols][N], missing flags and the pruned root.
int oracle_encode(const pacc_model* model, const pacc_opts* opts, const uint8_t* bases, int32_t length,
                  int8_t* tg_out, int32_t* n_cols, uint8_t* missing_out, int32_t* root_out, int32_t* filtered) {
    Model M;
    if (!build_model(model, opts, M)) return PACC_EINVAL;
    Element E(M);
    bool f = E.construct(0, bases, length);
    *filtered = f ? 1 : 0;
    if (f) { *n_cols = 0; return PACC_OK; }
    *n_cols = E.GG;
    for (size_t i = 0; i < (size_t)E.GG * M.N; i++) tg_out[i] = (int8_t)E.Tg[i];
    for (int s = 0; s < M.N; s++) missing_out[s] = (uint8_t)E.missing[s];
    *root_out = E.root;
    return PACC_OK;
}

// Per-column log-likelihood for a fixed Z and rates (Update_Tg(..., false)
// over all columns with every node unvisited, bpp_c.cpp:647-671, and
// log_exp_sum at the root).  z: [N] int32.
int oracle_loglik(const pacc_model* model, const pacc_opts* opts, const uint8_t* bases, int32_t length,
                  const int32_t* z, double c_rate, double n_rate, double* out, int32_t* n_cols) {
    Model M;
    if (!build_model(model, opts, M)) return PACC_EINVAL;
    pacc_opts o2 = *opts;
    o2.init_conserve_rate = c_rate;
    o2.init_acce_rate = n_rate;
    M.o = o2;
    Element E(M);
    if (E.construct(0, bases, length)) { *n_cols = 0; return PACC_FILTERED; }
    E.initMCMC(1);
    for (int s = 0; s < M.N; s++) E.Z[s] = z[s];
    std::vector<char> visited(M.N, 0);
    for (int g = 0; g < E.GG; g++) {
        E.Update_Tg(g, visited, false);
        out[g] = log_exp_sum(E.lamv(g, E.root), K);
    }
    *n_cols = E.GG;
    return PACC_OK;
}

// P^T matrices (bpp.hpp:375-380) for branch lengths d[i] and rates r[i]; [n][16].
int oracle_pmatrix(const pacc_model* model, const pacc_opts* opts, int n, const double* d, const double* r,
                   double* out) {
    Model M;
    if (!build_model(model, opts, M)) return PACC_EINVAL;
    for (int i = 0; i < n; i++) {
        Mat4 L = log_tm(M, d[i], r[i], true);
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++) out[i * 16 + a * 4 + b] = std::exp(L.a[a][b]);
    }
    return PACC_OK;
}

// Stream words, for known-answer tests of the generator.
void oracle_stream(uint32_t seed, uint64_t w0, int n, uint32_t* out) {
    oracle_rng::Stream st;
    st.set(seed);
    for (int i = 0; i < n; i++) out[i] = st.word_at(w0 + (uint64_t)i);
}

void oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    oracle_rng::philox4x32_10(ctr, key, out);
}

// Samplers on a fresh stream, for distribution tests.
void oracle_sample_gamma(uint32_t seed, double a, double b, int n, double* out) {
    oracle_rng::Stream st;
    st.set(seed);
    for (int i = 0; i < n; i++) out[i] = st.gamma(a, b);
}
void oracle_sample_beta(uint32_t seed, double a, double b, int n, double* out) {
    oracle_rng::Stream st;
    st.set(seed);
    for (int i = 0; i < n; i++) out[i] = st.beta(a, b);
}
void oracle_sample_categorical(uint32_t seed, int K_, const double* p, int n, int32_t* out) {
    oracle_rng::Stream st;
    st.set(seed);
    for (int i = 0; i < n; i++) out[i] = st.categorical(K_, p);
}

int oracle_eigen(const double* Q, double* lam, double* V, double* Vinv) {
    return pacc_eigen::decompose(4, Q, lam, V, Vinv);
}

}  // extern "C"
