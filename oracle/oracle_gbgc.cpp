// oracle_gbgc.cpp — TEST INFRASTRUCTURE (the oracle), never product code.
//
// A CPU restatement of the likelihood engine of PhyloAcc-ST-GBGC (the gBGC
// model), in the reference's log-space arithmetic and operation order:
//   * per-element column encoding, missing taxa and the collapse of the
//     missing outgroup path (BPP_C constructor, src/PhyloAcc-ST-GBGC/SRC/
//     bpp_c.hpp:143-379; getSubtree_missing, bpp_c.cpp:53-111);
//   * the rate matrix under selection s and GC bias b (getRate,
//     bpp_c.cpp:13-30) and the six per-branch log transition matrices of
//     init_cache_TM (bpp_c.cpp:1563-1621): classes 2 Z + B with Z in {0 null,
//     1 conserved, 2 accelerated} and B the gBGC flag;
//   * the log-space pruning pass of Update_Tg (bpp_c.cpp:477-540) and its
//     per-column log-likelihood (log_exp_sum, bpp.hpp:466-474);
//   * the expected (child base, parent base) counts of the sampling pass of
//     Update_Tg (bpp_c.cpp:541-596), the variational posterior_Tg_next.
// Armadillo's eig_gen/inv are replaced by eigen4.h, as in the stand-in build of
// the reference that pins this file (tests/golden/gbgc_engine).  Sums run in
// increasing index order; the max of a matrix is its first element then
// strict '>' comparisons (column-major scan), as the stand-in does.
#include "../include/pacc.h"
#include "../phyloacc_gb300/csrc/eigen4.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <set>
#include <vector>

#include "oracle_rng.h"

namespace {

typedef double M4[4][4];

// max of a 4x4 matrix scanned column-major (the stand-in's Mat::max)
double mat_max(const M4& a) {
    double m = a[0][0];
    for (int j = 0; j < 4; j++)
        for (int i = 0; i < 4; i++)
            if (a[i][j] > m) m = a[i][j];
    return m;
}

// log_multi (bpp.hpp:414-431): log of X^T y with log-space X and y
void log_multi(const M4& lx, const double* ly, double* out) {
    M4 a;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) a[i][j] = lx[i][j] + ly[i];
    const double mx = mat_max(a);
    if (mx == -INFINITY) {
        for (int j = 0; j < 4; j++) out[j] = -INFINITY;
        return;
    }
    for (int j = 0; j < 4; j++) {
        double s = 0;
        for (int i = 0; i < 4; i++) s += std::exp(a[i][j] - mx);
        out[j] = std::log(s) + mx;
    }
}

// log_exp_sum (bpp.hpp:466-474) of a 4-vector
double log_exp_sum4(const double* y) {
    double mx = y[0];
    for (int i = 1; i < 4; i++)
        if (y[i] > mx) mx = y[i];
    if (mx == -INFINITY) return -INFINITY;
    double s = 0;
    for (int i = 0; i < 4; i++) s += std::exp(y[i] - mx);
    return std::log(s) + mx;
}

// getRate (bpp_c.cpp:13-30): Q0 scaled entrywise by f(s + b B_ij) with
// f(x) = x / (1 - e^-x) (1 at 0), B = +1 for A/T -> C/G, -1 for C/G -> A/T,
// then the diagonal reset so that rows sum to zero
void get_rate(const double* Q0, double s, double b, M4& Q) {
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) Q[i][j] = Q0[i * 4 + j];
    if (s == 0 && b == 0) return;
    M4 B = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
    B[0][1] = b; B[0][2] = b; B[3][1] = b; B[3][2] = b;
    B[1][0] = -b; B[1][3] = -b; B[2][0] = -b; B[2][3] = -b;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            const double v = B[i][j] + s;
            B[i][j] = (v == 0) ? 1.0 : v / (1 - std::exp(-v));
        }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) Q[i][j] *= B[i][j];
    double c[4];
    for (int i = 0; i < 4; i++) {
        double t = 0;
        for (int j = 0; j < 4; j++) t += Q[i][j];
        c[i] = t;
    }
    for (int i = 0; i < 4; i++) Q[i][i] -= c[i];
}

// eig_gen + the transposes and inverse of init_cache_TM (bpp_c.cpp:1571-1584)
struct Eig {
    double lam[4];
    M4 vec;    // eigenvec = real(V)^T
    M4 inv;    // eigeninv = inv(eigenvec)
};
bool eig_of(const M4& Q, Eig& e) {
    double A[16], V[16], Vi[16], lam[4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) A[i * 4 + j] = Q[i][j];
    if (pacc_eigen::decompose(4, A, lam, V, Vi) != pacc_eigen::EIG_OK) return false;
    double T[16], Ti[16];
    for (int i = 0; i < 4; i++) {
        e.lam[i] = lam[i];
        for (int j = 0; j < 4; j++) T[i * 4 + j] = V[j * 4 + i];
    }
    if (pacc_eigen::invert(4, T, Ti) != pacc_eigen::EIG_OK) return false;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            e.vec[i][j] = T[i * 4 + j];
            e.inv[i][j] = Ti[i * 4 + j];
        }
    return true;
}

// log(eigeninv * (eigenvec with row i scaled by exp(lambda_i d))) (bpp_c.cpp:1593-1597)
void log_transition(const Eig& e, double d, M4& out) {
    M4 x;
    for (int i = 0; i < 4; i++) {
        const double t = std::exp(e.lam[i] * d);
        for (int j = 0; j < 4; j++) x[i][j] = e.vec[i][j] * t;
    }
    for (int a = 0; a < 4; a++)
        for (int b = 0; b < 4; b++) {
            double s = 0;
            for (int k = 0; k < 4; k++) s += e.inv[a][k] * x[k][b];
            out[a][b] = std::log(s);
        }
}

struct Elem {
    int S, N, GG, root;
    std::vector<int> c0, c1, parent;
    std::vector<double> dist;
    std::vector<char> missing;
    std::vector<int> nodes;              // postorder from the (moved) root
    std::vector<std::vector<double>> lam;   // [GG][N*4] log partials
};

// getSubtree_missing (bpp_c.cpp:53-111): collapse missing branches on the
// outgroup path, moving the root down
void subtree_missing(Elem& E, const std::set<int>& upper, int ss, int child) {
    if (upper.find(ss) == upper.end() || ss < E.S) return;
    int s = ss;
    while (upper.find(s) != upper.end() && s >= E.S) {
        const int p0 = E.c0[s], p1 = E.c1[s];
        if (E.missing[p0] && !E.missing[p1]) {
            E.parent[p0] = -1;
            E.dist[p1] += E.dist[s];
            if (s == E.root) {
                E.root = p1;
            } else {
                if (child == 0) E.c0[E.parent[ss]] = p1; else E.c1[E.parent[ss]] = p1;
                E.parent[p1] = E.parent[ss];
            }
            s = p1;
        } else if (!E.missing[p0] && E.missing[p1]) {
            E.parent[p1] = -1;
            E.dist[p0] += E.dist[s];
            if (s == E.root) {
                E.root = p0;
            } else {
                if (child == 0) E.c0[E.parent[ss]] = p0; else E.c1[E.parent[ss]] = p0;
                E.parent[p0] = E.parent[ss];
            }
            s = p0;
        } else {
            subtree_missing(E, upper, E.c0[s], 0);
            subtree_missing(E, upper, E.c1[s], 1);
            return;
        }
    }
}

void postorder(const Elem& E, int j, std::vector<int>& out) {
    if (E.c0[j] != -1) postorder(E, E.c0[j], out);
    if (E.c1[j] != -1) postorder(E, E.c1[j], out);
    out.push_back(j);
}

// The BPP_C constructor of the gBGC model (bpp_c.hpp:153-379): leaf
// partials, missing taxa, the conserved-species filter (true: filtered), the
// outgroup path (getUppertree, bpp.cpp:454-476) and its collapse
// (getSubtree_missing), and the postorder of the element's tree.
bool setup_element(const pacc_model* m, const uint8_t* bases, int32_t GG, int32_t gapchar, double missing_thres,
                   double conserve_prop, Elem& E, std::set<int>& upper) {
    E.S = m->n_species;
    E.N = 2 * E.S - 1;
    E.GG = GG;
    const int S = E.S, N = E.N;
    E.c0.assign(N, -1); E.c1.assign(N, -1); E.parent.assign(N, -1);
    E.dist.assign(m->distances, m->distances + N);
    for (int i = 0; i < N; i++) {
        E.c0[i] = m->children[2 * i];
        E.c1[i] = m->children[2 * i + 1];
        if (E.c0[i] >= 0) E.parent[E.c0[i]] = i;
        if (E.c1[i] >= 0) E.parent[E.c1[i]] = i;
    }
    E.root = N - 1;
    // leaf partials (bpp_c.hpp:203-251)
    E.lam.assign(GG, std::vector<double>((size_t)N * 4, 0.0));
    std::vector<int> num_missing(S, 0);
    for (int s = 0; s < S; s++) {
        const uint8_t* y = bases + (size_t)s * GG;
        for (int g = 0; g < GG; g++) {
            double* l = &E.lam[g][(size_t)s * 4];
            for (int k = 0; k < 4; k++) l[k] = -INFINITY;
            if ((int)y[g] == gapchar) num_missing[s]++;
            switch ((char)y[g]) {
                case 'a': l[0] = 0; break;
                case 'c': l[1] = 0; break;
                case 'g': l[2] = 0; break;
                case 't': l[3] = 0; break;
                case 'r': l[0] = 0; l[2] = 0; break;
                case 'y': l[1] = 0; l[3] = 0; break;
                case 'k': l[2] = 0; l[3] = 0; break;
                case 'm': l[0] = 0; l[1] = 0; break;
                case 's': l[1] = 0; l[2] = 0; break;
                case 'w': l[0] = 0; l[3] = 0; break;
                default: for (int k = 0; k < 4; k++) l[k] = 0;   // '-' (four bases) and the rest
            }
        }
    }
    // missing (bpp_c.hpp:269-292)
    E.missing.assign(N, 0);
    for (int s = S; s < N; s++) {
        const int p[2] = {E.c0[s], E.c1[s]};
        for (int cc = 0; cc < 2; cc++)
            if (p[cc] < S && num_missing[p[cc]] > missing_thres * GG) E.missing[p[cc]] = 1;
        if (E.missing[p[0]] && E.missing[p[1]]) E.missing[s] = 1;
    }
    int ct = 0;
    for (int i = 0; i < m->n_conserve; i++)
        if (m->conserve[i] >= 0 && m->conserve[i] < N && E.missing[m->conserve[i]]) ct++;
    if (ct > conserve_prop * m->n_conserve) return true;
    // the outgroup path (getUppertree, bpp.cpp:454-476) and its collapse
    upper.clear();
    for (int i = 0; i < m->n_outgroup; i++) {
        int p = m->outgroup[i];
        while (p != N - 1 && p >= 0 && p < N) { upper.insert(p); p = E.parent[p]; }
    }
    upper.insert(N - 1);
    subtree_missing(E, upper, N - 1, -1);
    E.parent[E.root] = N;
    postorder(E, E.root, E.nodes);
    return false;
}


// ---------------------------------------------------------------------------
// The gBGC chain of one element: BPP_C's initMCMC, Gibbs, Eval2 and
// Output_init (bpp_c.cpp:120-452,477-1137,1563-1764; bpp_c2.cpp:29-286,
// 287-500,603-660) for the three models M0, M2, M1, drawn in that order from
// one stream seeded with SEED (main.cpp:383-412).  Class index k = Z + 3 B
// throughout: 0 null, 1 cons, 2 neut, 3 null+B, 4 cons+B, 5 neut+B (the
// reference's log_cache_TM_* vectors, log_emission and log_prob_back slots).
// ---------------------------------------------------------------------------
struct Mat4 { M4 a; };
typedef std::array<double, 6> V6;
struct TM63 { double a[6][3]; };

// log_multi (bpp.hpp:414-431) of the 6x3 log_TM_Int by a 6-vector
void log_multi63(const double (*lx)[3], const V6& ly, double* out) {
    double a[6][3];
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 3; j++) a[i][j] = lx[i][j] + ly[i];
    double mx = a[0][0];
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 6; i++)
            if (a[i][j] > mx) mx = a[i][j];
    if (mx == -INFINITY) {
        for (int j = 0; j < 3; j++) out[j] = -INFINITY;
        return;
    }
    for (int j = 0; j < 3; j++) {
        double t = 0;
        for (int i = 0; i < 6; i++) t += std::exp(a[i][j] - mx);
        out[j] = std::log(t) + mx;
    }
}

double gamma_pdf(double x, double a, double b) {   // the GSL density's definition
    if (x < 0) return 0.0;
    if (x == 0) return (a == 1) ? 1.0 / b : 0.0;
    return std::exp((a - 1) * std::log(x) - x / b - std::lgamma(a) - a * std::log(b));
}

double accu_prod(const M4& a, const M4& b) {   // accu(a % b), column-major
    double t = 0;
    for (int j = 0; j < 4; j++)
        for (int i = 0; i < 4; i++) t += a[i][j] * b[i][j];
    return t;
}

struct GChain {
    const pacc_model* m;
    const pacc_gbgc_opts* o;
    Elem& E;
    const std::set<int>& upper;
    oracle_rng::Stream rng;
    int S, N, GG, root, T, burn, mcmc;
    std::vector<int> upper_c, fixZ, Z;
    std::vector<char> B;
    std::vector<Mat4> cache[6];
    std::vector<TM63> lTM;   // [N] 6 x 3 log Z-transition (rows: child Z + 3B, cols: parent Z)
    std::vector<V6> emis, lpb;
    std::vector<std::vector<double>> msg;         // [GG][N*4]
    std::vector<Mat4> post, post_next;
    double log_pi[4];
    std::vector<double> tr_loglik, tr_full, tr_n, tr_c, tr_gb;
    std::vector<std::vector<int>> tr_Z;
    std::vector<std::vector<char>> tr_B;
    double logpZC = 0, logp_Z = 0, MaxLoglik = -INFINITY;
    std::vector<int> Max_Z;
    std::vector<char> Max_B;
    int Max_m = 0, m_it = 0;

    GChain(const pacc_model* m_, const pacc_gbgc_opts* o_, Elem& E_, const std::set<int>& up)
        : m(m_), o(o_), E(E_), upper(up) {
        S = E.S; N = E.N; GG = E.GG; root = E.root;
        burn = o->burnin; mcmc = o->mcmc; T = burn + mcmc;
        rng.set(o->seed);
        for (int s : E.nodes)
            if (upper.count(s)) upper_c.push_back(s);
        for (int k = 0; k < 6; k++) cache[k].assign(N, Mat4{});
        for (int k = 0; k < 6; k++)
            for (int s = 0; s < N; s++) std::memset(cache[k][s].a, 0, sizeof(M4));
        // TM_Int / log_TM_Int (bpp.hpp:278-324), the outgroup path kept at Z <= 1
        lTM.resize(N);
        for (int s = 0; s < N; s++) {
            double tm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            tm[0][0] = 1 - o->prep_grate;
            tm[1][0] = o->prep_grate;
            tm[1][1] = 1 - o->prep_lrate;
            tm[2][1] = o->prep_lrate;
            tm[2][2] = 1;
            if (upper.count(s)) { tm[1][1] = 1; tm[2][1] = 0; }
            for (int r = 0; r < 6; r++)
                for (int c = 0; c < 3; c++) lTM[s].a[r][c] = std::log(tm[r % 3][c]);
        }
        msg.assign(GG, std::vector<double>((size_t)N * 4, 0.0));
        post.assign(N, Mat4{});
        post_next.assign(N, Mat4{});
        for (int s = 0; s < N; s++) {
            std::memset(post[s].a, 0, sizeof(M4));
            std::memset(post_next[s].a, 0, sizeof(M4));
        }
        for (int i = 0; i < 4; i++) log_pi[i] = std::log(m->pi[i]);
        tr_loglik.assign(T, 0); tr_full.assign(T, 0); tr_n.assign(T, 0); tr_c.assign(T, 0); tr_gb.assign(T, 0);
        tr_Z.assign(T, std::vector<int>(N, 1));
        tr_B.assign(T, std::vector<char>(N, 0));
    }

    void up_pass(bool half) {   // message passing bottom-up over log_prob_back
        for (size_t it = 0; it + 1 < E.nodes.size(); it++) {
            const int s = E.nodes[it], p = E.parent[s];
            double r[3];
            log_multi63(lTM[s].a, lpb[s], r);
            for (int j = 0; j < 3; j++) {
                const double t = half ? r[j] - std::log(2.0) : r[j];
                lpb[p][j] += t;
                lpb[p][3 + j] += t;
            }
        }
    }

    bool set_caches(const double* Q0, const double* sel, const double* bias, int n, const int* cls, std::vector<Mat4>* dst,
                    bool skip_neut_fixed) {
        Eig eg[6];
        for (int i = 0; i < n; i++) {
            M4 Q;
            get_rate(Q0, sel[i], bias[i], Q);
            if (!eig_of(Q, eg[i])) return false;
        }
        for (size_t it = 0; it + 1 < E.nodes.size(); it++) {
            const int s = E.nodes[it];
            if (E.missing[s]) continue;
            for (int i = 0; i < n; i++) {
                if (skip_neut_fixed && cls[i] % 3 == 2 && fixZ[s] == 1) continue;
                log_transition(eg[i], E.dist[s], dst[i][s].a);
            }
        }
        return true;
    }

    // initMCMC (bpp_c.cpp:120-257), first chain
    bool init(int resZ) {
        B.assign(N, 0);
        // the first chain: -1 off the element's tree, 0 on it; a later chain
        // takes bpp.cur_Z, all zeros without SAMPLE_HYPER (bpp_c.cpp:124-135)
        Z.assign(N, o->chain > 0 ? 0 : -1);
        for (int s : E.nodes) Z[s] = 0;
        Z[root] = 0;
        fixZ.assign(N, -1);
        for (int s : upper_c) fixZ[s] = 1;
        fixZ[root] = 0;
        if (resZ == 2) {
            for (int s = 0; s < S; s++) fixZ[s] = 1;
            for (int i = 0; i < o->n_target; i++)
                if (o->target[i] >= 0 && o->target[i] < N) fixZ[o->target[i]] = -1;
        } else if (resZ == 0) {
            for (size_t it = 0; it + 1 < E.nodes.size(); it++) fixZ[E.nodes[it]] = 1;
        }
        MaxLoglik = -INFINITY;
        tr_n[0] = o->acce_rate;
        tr_c[0] = o->conserve_rate;
        tr_gb[0] = o->init_gc;
        const double sel[6] = {0, tr_c[0], tr_n[0], 0, tr_c[0], tr_n[0]};
        const double bias[6] = {0, 0, 0, tr_gb[0], tr_gb[0], tr_gb[0]};
        const int cls[6] = {0, 1, 2, 3, 4, 5};
        // Qs[0] is the rate matrix itself (getRate returns Q0 at s = b = 0)
        if (!set_caches(m->rate_matrix, sel, bias, 6, cls, cache, true)) return false;
        lpb.assign(N, V6{0, 0, 0, 0, 0, 0});
        emis.assign(N, V6{0, 0, 0, 0, 0, 0});
        const double lnc = std::log(o->ncons_to_mis), lc = std::log(o->cons_to_mis);
        for (size_t it = 0; it + 1 < E.nodes.size(); it++) {
            const int s = E.nodes[it], p = E.parent[s];
            if (E.missing[p]) continue;
            if (E.missing[s]) emis[s] = V6{lnc, lc, lnc, lnc, lc, lnc};
        }
        for (int s = 0; s < N; s++)
            if (fixZ[s] == 1) {
                lpb[s][2] = lpb[s][5] = -INFINITY;
                emis[s][2] = emis[s][5] = -INFINITY;
            }
        up_pass(true);
        logpZC = lpb[root][0];
        return true;
    }

    const M4& cls_mat(int s) const { return cache[Z[s] + (B[s] ? 3 : 0)][s].a; }

    // Update_Tg without sampling (bpp_c.cpp:480-540) over every column; returns
    // sum_g log_exp_sum(lambda root)
    double prune_all() {
        double tot = 0;
        for (int g = 0; g < GG; g++) {
            std::vector<double>& L = E.lam[g];
            for (int s = S; s < N; s++)
                for (int j = 0; j < 4; j++) L[(size_t)s * 4 + j] = 0;
            for (int s : E.nodes) {
                if (s < S || E.missing[s]) continue;
                const int p[2] = {E.c0[s], E.c1[s]};
                for (int cc = 0; cc < 2; cc++) {
                    const int chi = p[cc];
                    if (E.missing[chi]) continue;
                    log_multi(cls_mat(chi), &L[(size_t)chi * 4], &msg[g][(size_t)chi * 4]);
                    for (int j = 0; j < 4; j++) L[(size_t)s * 4 + j] += msg[g][(size_t)chi * 4 + j];
                }
            }
            for (int j = 0; j < 4; j++) L[(size_t)root * 4 + j] += log_pi[j];
            tot += log_exp_sum4(&L[(size_t)root * 4]);
        }
        return tot;
    }

    // Update_Tg with sampling (bpp_c.cpp:541-596): expected counts into post_next
    void counts_all() {
        for (int s : E.nodes) std::memset(post_next[s].a, 0, sizeof(M4));
        std::vector<double> ltp((size_t)N * 4);
        for (int g = 0; g < GG; g++) {
            const std::vector<double>& L = E.lam[g];
            const double* lr = &L[(size_t)root * 4];
            double prob[4];
            const double x = log_exp_sum4(lr);
            for (int j = 0; j < 4; j++) prob[j] = (x == INFINITY) ? 0.0 : std::exp(lr[j] - x);
            std::fill(ltp.begin(), ltp.end(), 0.0);
            for (int j = 0; j < 4; j++) {
                post_next[root].a[j][0] += prob[j];
                ltp[(size_t)root * 4 + j] = std::log(prob[j]);
            }
            for (int it = (int)E.nodes.size() - 2; it >= 0; it--) {
                const int s = E.nodes[it], pa = E.parent[s];
                if (E.missing[s]) continue;
                const M4& P = cls_mat(s);
                M4 tp;
                for (int i = 0; i < 4; i++)
                    for (int j = 0; j < 4; j++) tp[i][j] = P[i][j] + (ltp[(size_t)pa * 4 + j] - msg[g][(size_t)s * 4 + j]);
                for (int i = 0; i < 4; i++)
                    for (int j = 0; j < 4; j++) tp[i][j] += L[(size_t)s * 4 + i];
                const double mx = mat_max(tp);
                for (int i = 0; i < 4; i++) {
                    double t = 0;
                    for (int j = 0; j < 4; j++) t += std::exp(tp[i][j] - mx);
                    ltp[(size_t)s * 4 + i] = std::log(t) + mx;
                }
                for (int i = 0; i < 4; i++)
                    for (int j = 0; j < 4; j++) post_next[s].a[i][j] += std::exp(tp[i][j]);
            }
        }
    }

    double prior_Z() const {   // prior_Z (bpp_c2.cpp:484-498)
        double r = 0;
        for (int it = (int)E.nodes.size() - 2; it >= 0; it--) {
            const int s = E.nodes[it], p = E.parent[s];
            r += lTM[s].a[Z[s]][Z[p]];
        }
        return r;
    }

    // initial_prob_back (bpp_c2.cpp:354-457)
    double initial_prob_back() {
        double elbo = 0;
        for (size_t it = 0; it + 1 < E.nodes.size(); it++) {
            const int s = E.nodes[it];
            if (E.missing[s]) continue;
            for (int i = 0; i < 6; i++) {
                if (fixZ[s] == 1 && i % 3 == 2) continue;
                emis[s][i] = accu_prod(cache[i][s].a, post[s].a);
                if (i == Z[s] + 3 * B[s]) elbo += emis[s][i];
                emis[s][i] += (i < 3) ? std::log(1 - o->gc_prior_c) : std::log(o->gc_prior_c);
                emis[s][i] += (i % 3 == 1) ? std::log(1 - o->cons_to_mis) : std::log(1 - o->ncons_to_mis);
            }
        }
        for (size_t it = 0; it + 1 < E.nodes.size(); it++) lpb[E.nodes[it]] = emis[E.nodes[it]];
        lpb[root] = V6{0, 0, 0, 0, 0, 0};
        up_pass(false);
        return elbo;
    }

    // integrate_ZB (bpp_c.cpp:1765-1799) with update_cache_TM and getEmission_update(-1)
    bool integrate_ZB(double nc, double nn, double ngb, std::vector<V6>& emis_tmp, std::vector<Mat4>* tmp) {
        const double sel[5] = {nc, nn, 0, nc, nn};
        const double bias[5] = {0, 0, ngb, ngb, ngb};
        const int cls[5] = {1, 2, 3, 4, 5};
        if (!set_caches(m->rate_matrix, sel, bias, 5, cls, tmp, true)) return false;
        for (size_t it = 0; it + 1 < E.nodes.size(); it++) {
            const int s = E.nodes[it];
            if (E.missing[s]) continue;
            for (int i = 0; i < 5; i++) {
                const int j = i + 1;
                if (fixZ[s] == 1 && j % 3 == 2) continue;
                emis_tmp[s][j] = accu_prod(tmp[i][s].a, post[s].a);
                emis_tmp[s][j] += (j < 3) ? std::log(1 - o->gc_prior_c) : std::log(o->gc_prior_c);
                emis_tmp[s][j] += (j % 3 == 1) ? std::log(1 - o->cons_to_mis) : std::log(1 - o->ncons_to_mis);
            }
        }
        for (size_t it = 0; it + 1 < E.nodes.size(); it++) lpb[E.nodes[it]] = emis_tmp[E.nodes[it]];
        lpb[root] = V6{0, 0, 0, 0, 0, 0};
        up_pass(false);
        return true;
    }

    void emission_update(bool accept, std::vector<V6>& emis_tmp, std::vector<Mat4>* tmp) {
        for (size_t it = 0; it + 1 < E.nodes.size(); it++) {
            const int s = E.nodes[it];
            if (E.missing[s]) continue;
            for (int i = 0; i < 5; i++) {
                const int j = i + 1;
                if (fixZ[s] == 1 && j % 3 == 2) continue;
                if (accept) {
                    emis[s][j] = emis_tmp[s][j];
                    cache[j][s] = tmp[i][s];
                } else {
                    emis_tmp[s][j] = emis[s][j];
                }
            }
        }
    }

    // sample_rates (bpp_c.cpp:881-976), M = 3 moves
    bool sample_rates(double& loglik_old, int resZ) {
        bool move = false;
        std::vector<V6> emis_tmp = emis;
        std::vector<Mat4> tmp[5];
        for (int i = 0; i < 5; i++) {
            tmp[i].assign(N, Mat4{});
            for (int s = 0; s < N; s++) std::memset(tmp[i][s].a, 0, sizeof(M4));
        }
        const int mm_ = m_it;
        double cur_gB = tr_gb[mm_], cur_rc = tr_c[mm_], cur_rn = tr_n[mm_];
        for (int mm = 0; mm < 3; mm++) {
            double u = (rng.uniform() - 0.5) * o->prop_gc * 2;
            double new_gB = cur_gB + u;
            if (new_gB < 0.01) new_gB = cur_gB;
            double new_n = cur_rn;
            if (resZ != 0) {
                u = rng.uniform() * (o->prop_n - 1 / o->prop_n) + 1 / o->prop_n;
                new_n = (cur_rn + o->acce_prior_shift) * u - o->acce_prior_shift;
            }
            u = rng.uniform() * (o->prop_c - 1 / o->prop_c) + 1 / o->prop_c;
            const double new_c = cur_rc * u;
            if (!integrate_ZB(new_c, new_n, new_gB, emis_tmp, tmp)) return false;
            double MH = lpb[root][0] - loglik_old + std::log(gamma_pdf(new_gB, o->gc_prior_a, o->gc_prior_b)) -
                        std::log(gamma_pdf(cur_gB, o->gc_prior_a, o->gc_prior_b));
            if (resZ != 0)
                MH += std::log(gamma_pdf(new_n + o->acce_prior_shift, o->acce_prior_a, o->acce_prior_b)) -
                      std::log(gamma_pdf(cur_rn + o->acce_prior_shift, o->acce_prior_a, o->acce_prior_b));
            MH += std::log(gamma_pdf(-new_c, o->conserve_prior_a, o->conserve_prior_b)) -
                  std::log(gamma_pdf(-cur_rc, o->conserve_prior_a, o->conserve_prior_b)) - std::log(-new_c) +
                  std::log(-cur_rc);
            if (std::log(rng.uniform()) < MH) {
                cur_gB = new_gB;
                cur_rn = new_n;
                cur_rc = new_c;
                loglik_old = lpb[root][0];
                emission_update(true, emis_tmp, tmp);
                move = true;
            } else {
                emission_update(false, emis_tmp, tmp);
            }
        }
        tr_c[mm_ + 1] = cur_rc;
        tr_n[mm_ + 1] = cur_rn;
        tr_gb[mm_ + 1] = cur_gB;
        return move;
    }

    // Update_ZB (bpp_c.cpp:1667-1763)
    int update_ZB() {
        for (size_t it = 0; it + 1 < E.nodes.size(); it++) lpb[E.nodes[it]] = emis[E.nodes[it]];
        lpb[root] = V6{0, 0, 0, 0, 0, 0};
        up_pass(false);
        int changed = 0;
        for (int it = (int)E.nodes.size() - 2; it >= 0; it--) {
            const int s = E.nodes[it], p = E.parent[s];
            const int old = Z[s];
            if (Z[p] != 2) {
                double x[6], w[6];
                for (int r = 0; r < 6; r++) x[r] = lTM[s].a[r][Z[p]] + lpb[s][r];
                double mx = x[0];
                for (int r = 1; r < 6; r++)
                    if (x[r] > mx) mx = x[r];
                for (int r = 0; r < 6; r++) w[r] = std::exp(x[r] - mx);
                const int nn = rng.categorical(6, w);
                Z[s] = nn % 3;
                if (!E.missing[s]) B[s] = nn > 2;
            } else {
                Z[s] = 2;
                double x[2] = {lpb[s][2], lpb[s][5]}, w[2];
                const double mx = x[1] > x[0] ? x[1] : x[0];
                for (int r = 0; r < 2; r++) w[r] = std::exp(x[r] - mx);
                const int nn = rng.categorical(2, w);
                if (!E.missing[s]) B[s] = nn > 0;
            }
            if (old != Z[s]) changed++;
        }
        return changed;
    }

    double ELBO() const {   // bpp_c.cpp:840-878
        double r = 0;
        for (size_t it = 0; it + 1 < E.nodes.size(); it++) {
            const int s = E.nodes[it];
            if (E.missing[s]) continue;
            r += accu_prod(cls_mat(s), post[s].a);
        }
        return r;
    }

    // update_rates (bpp_c.cpp:1079-1137), not adaptive
    bool update_rates(double elbo_old) {
        const int mm = m_it;
        const int changed = update_ZB();
        std::vector<std::vector<double>> lam0 = E.lam, msg0 = msg;
        const double loglik_new = prune_all();
        const double elbo_new = ELBO();
        const double MH = loglik_new - tr_loglik[mm] + elbo_old - elbo_new;
        if (std::log(rng.uniform()) < MH) {
            tr_loglik[mm + 1] = loglik_new;
            if (changed > 0) logp_Z = prior_Z() - logpZC;
            return true;
        }
        tr_c[mm + 1] = tr_c[mm];
        tr_n[mm + 1] = tr_n[mm];
        tr_gb[mm + 1] = tr_gb[mm];
        E.lam = lam0;
        msg = msg0;
        Z = tr_Z[mm];
        B = tr_B[mm];
        return false;
    }

    // MonitorChain (bpp_c.cpp:598-699)
    void monitor(int mm, bool move_r, int resZ, const std::vector<double>& root_ll) {
        if (mm == 0) {
            tr_loglik[0] = 0;
            for (int g = 0; g < GG; g++) tr_loglik[0] += root_ll[g];
        }
        if (!move_r) {
            tr_loglik[mm] = tr_loglik[mm - 1];
            tr_full[mm] = tr_full[mm - 1];
        } else {
            tr_full[mm] = tr_loglik[mm] + logp_Z;
            tr_full[mm] += std::log(gamma_pdf(-tr_c[mm], o->conserve_prior_a, o->conserve_prior_b));
            if (resZ != 0)
                tr_full[mm] += std::log(gamma_pdf(tr_n[mm] + o->acce_prior_shift, o->acce_prior_a, o->acce_prior_b));
            int gb = 0, ungb = 0, mz[4] = {0, 0, 0, 0};
            for (size_t it = 0; it + 1 < E.nodes.size(); it++) {
                const int s = E.nodes[it], p = E.parent[s];
                if (E.missing[p]) continue;
                mz[2 * (E.missing[s] ? 1 : 0) + (Z[s] == 1 ? 1 : 0)] += 1;
                if (E.missing[s]) continue;
                if (B[s]) gb++; else ungb++;
            }
            tr_full[mm] += std::log(1 - o->ncons_to_mis) * mz[0] + std::log(1 - o->cons_to_mis) * mz[1] +
                           std::log(o->ncons_to_mis) * mz[2] + std::log(o->cons_to_mis) * mz[3];
            tr_full[mm] += std::log(1 - o->gc_prior_c) * ungb +
                           std::log(gamma_pdf(tr_gb[mm], o->gc_prior_a, o->gc_prior_b)) + std::log(o->gc_prior_c) * gb;
        }
        tr_Z[mm] = Z;
        tr_B[mm] = B;
        if (mm >= burn && tr_full[mm] > MaxLoglik) {
            MaxLoglik = tr_full[mm];
            Max_Z = Z;
            Max_B = B;
            Max_m = mm;
        }
    }

    // Gibbs (bpp_c.cpp:259-349)
    bool gibbs(int resZ) {
        std::vector<double> root_ll(GG);
        prune_all();
        for (int g = 0; g < GG; g++) root_ll[g] = log_exp_sum4(&E.lam[g][(size_t)root * 4]);
        logp_Z = prior_Z() - logpZC;
        bool move_r = true;
        for (int mm = 0; mm < T; mm++) {
            m_it = mm;
            monitor(mm, move_r, resZ, root_ll);
            if (mm == T - 1) break;
            if (move_r) counts_all();
            if (mm == 0) post = post_next;
            const double elbo_old = initial_prob_back();
            double loglik_old = lpb[root][0];
            std::vector<Mat4> saved[6];
            for (int k = 1; k < 6; k++) saved[k] = cache[k];
            sample_rates(loglik_old, resZ);
            move_r = update_rates(elbo_old);
            if (!move_r)
                for (int k = 1; k < 6; k++) cache[k] = saved[k];
            post = post_next;
        }
        return true;
    }

    std::set<int> shifts(const std::vector<char>& b) const {   // getShifts (bpp_c2.cpp:14-27)
        std::set<int> r;
        for (int s : E.nodes)
            if (!E.missing[s] && b[s]) r.insert(s);
        return r;
    }

    // Eval2 (bpp_c2.cpp:29-286): the model's marginal log-likelihood
    double eval2(int resZ) {
        Z = Max_Z;
        std::vector<int> uncertain;
        for (int s = 0; s < N; s++) {
            int c = 0;
            for (int i = burn; i < T; i++)
                if (tr_Z[i][s] == Max_Z[s]) c++;
            if (c < mcmc) uncertain.push_back(s);
        }
        const int d = 2 + (resZ != 0 ? 1 : 0);
        std::vector<std::vector<int>> configZ(1, Max_Z);
        std::vector<int> nZ(1, 0);
        std::vector<std::vector<std::set<int>>> cZB(1);
        std::vector<std::vector<int>> nZB(1);
        std::vector<std::vector<double>> means(1, std::vector<double>(d, 0.0));
        std::vector<std::vector<double>> var(1, std::vector<double>(d * d, 0.0));   // column-major d x d
        std::vector<double> sumf(1, 0.0);
        for (int i = T - 1; i >= burn; i--) {
            size_t j = 0;
            for (; j < configZ.size(); j++) {
                size_t u = 0;
                for (; u < uncertain.size(); u++)
                    if (tr_Z[i][uncertain[u]] != configZ[j][uncertain[u]]) break;
                if (u == uncertain.size()) break;
            }
            if (j == configZ.size()) {
                configZ.push_back(tr_Z[i]);
                nZ.push_back(0);
                cZB.emplace_back();
                nZB.emplace_back();
                means.emplace_back(d, 0.0);
                var.emplace_back(d * d, 0.0);
                sumf.push_back(0.0);
            }
            nZ[j]++;
            const std::set<int> ts = shifts(tr_B[i]);
            size_t k = 0;
            for (; k < cZB[j].size(); k++)
                if (ts == cZB[j][k]) break;
            if (k == cZB[j].size()) {
                cZB[j].push_back(ts);
                nZB[j].push_back(0);
            }
            nZB[j][k]++;
            auto V = [&](int r, int c) -> double& { return var[j][c * d + r]; };
            V(1, 1) += tr_c[i] * tr_c[i];
            means[j][1] += tr_c[i];
            V(0, 0) += tr_gb[i] * tr_gb[i];
            means[j][0] += tr_gb[i];
            V(0, 1) += tr_c[i] * tr_gb[i];
            if (resZ != 0) {
                V(2, 2) += tr_n[i] * tr_n[i];
                means[j][2] += tr_n[i];
                V(1, 2) += tr_c[i] * tr_n[i];
                V(0, 2) += tr_gb[i] * tr_n[i];
            }
            sumf[j] += tr_full[i];
        }
        auto cov = [&](const std::vector<double>& v, const std::vector<double>& mu, double n) {
            std::vector<double> t(d * d);
            for (int c = 0; c < d; c++)
                for (int r = 0; r < d; r++) t[c * d + r] = (r > c) ? v[r * d + c] : v[c * d + r];   // symmatu
            for (int c = 0; c < d; c++)
                for (int r = 0; r < d; r++) t[c * d + r] -= mu[r] * mu[c] / n;
            for (int q = 0; q < d * d; q++) t[q] /= (n - 1);
            return t;
        };
        auto log_det = [&](std::vector<double> u, double& val, double& sign) {   // LU with partial pivoting
            sign = 1.0;
            val = 0.0;
            for (int k = 0; k < d; k++) {
                int p = k;
                for (int i = k + 1; i < d; i++)
                    if (std::fabs(u[k * d + i]) > std::fabs(u[k * d + p])) p = i;
                if (p != k) {
                    for (int j = 0; j < d; j++) std::swap(u[j * d + k], u[j * d + p]);
                    sign = -sign;
                }
                const double piv = u[k * d + k];
                if (piv == 0) { val = -INFINITY; sign = 0; return; }
                if (piv < 0) sign = -sign;
                val += std::log(std::fabs(piv));
                for (int i = k + 1; i < d; i++) {
                    const double f = u[k * d + i] / piv;
                    for (int j = k; j < d; j++) u[j * d + i] -= f * u[j * d + k];
                }
            }
        };
        auto logdiag = [&](const std::vector<double>& t) {
            double r = 0;
            for (int q = 0; q < d; q++) r += std::log(t[q * d + q]);
            return r;
        };
        double VB = 0, logdet = 0, sign = 1;
        int eff = 0;
        for (size_t i = 0; i < configZ.size(); i++) {
            const double w = (double)nZ[i] / mcmc;
            if (w < 0.05) continue;
            const std::vector<double> tv = cov(var[i], means[i], (double)nZ[i]);
            if (nZ[i] > 10) log_det(tv, logdet, sign);
            if (nZ[i] <= 10 || sign < 0) logdet = logdiag(tv);
            if (logdet == -INFINITY) continue;
            eff += nZ[i];
            double tB = 0;
            for (int c : nZB[i]) tB += (double)c * std::log((double)c);
            VB -= tB;
            VB += (double)(nZ[i] - 1) / 2 * d;
            VB += sumf[i];
            VB += 0.5 * logdet * nZ[i];
        }
        if (eff == 0) {
            std::vector<double> mean0(d, 0.0), var0(d * d, 0.0);
            VB = 0;
            double tB = 0;
            for (size_t i = 0; i < configZ.size(); i++) {
                for (int q = 0; q < d; q++) mean0[q] += means[i][q];
                for (int q = 0; q < d * d; q++) var0[q] += var[i][q];
                VB += sumf[i];
                for (int c : nZB[i]) tB += (double)c * std::log((double)c);
            }
            VB -= tB;
            const std::vector<double> tv = cov(var0, mean0, (double)mcmc);
            log_det(tv, logdet, sign);
            if (sign < 0) logdet = logdiag(tv);
            if (logdet != -INFINITY) {
                VB += 0.5 * logdet * mcmc;
                VB += (double)(mcmc - 1) / 2 * d;
                eff = mcmc;
            }
        }
        const double tail = (double)d / 2 * std::log(2 * M_PI);
        if (resZ == 1 && eff == 0) return MaxLoglik;
        return VB / eff + std::log((double)eff) + tail;
    }

    // Output_init (bpp_c2.cpp:603-660): medians of the rates, B and Z frequencies
    void output(int resZ, pacc_gbgc_result* r, int slot) {
        auto med = [&](std::vector<double> v) {
            std::sort(v.begin() + burn, v.end());
            return v[v.size() / 2];
        };
        r->rates[slot][0] = med(tr_n);
        r->rates[slot][1] = med(tr_c);
        r->rates[slot][2] = med(tr_gb);
        (void)resZ;
        for (int s = 0; s < N; s++) {
            int cz[4] = {0, 0, 0, 0}, cb = 0;
            for (int i = burn; i < T; i++) {
                cz[tr_Z[i][s] + 1]++;
                cb += tr_B[i][s];
            }
            if (E.missing[s]) cz[0] = mcmc;
            if (r->post_b) r->post_b[(size_t)slot * N + s] = (double)cb / mcmc;
            if (r->post_z)
                for (int k = 0; k < 4; k++) r->post_z[((size_t)slot * N + s) * 4 + k] = (double)cz[k] / mcmc;
            if (r->max_z) r->max_z[(size_t)slot * N + s] = Max_Z[s];
            if (r->max_b) r->max_b[(size_t)slot * N + s] = (int8_t)Max_B[s];
        }
        if (r->trace) {
            const int W = 4 + 2 * N;
            for (int i = 0; i < T; i++) {
                double* row = r->trace + ((size_t)slot * T + i) * W;
                row[0] = tr_full[i]; row[1] = tr_n[i]; row[2] = tr_c[i]; row[3] = tr_gb[i];
                for (int s = 0; s < N; s++) {
                    row[4 + s] = tr_B[i][s];
                    row[4 + N + s] = tr_Z[i][s];
                }
            }
        }
    }
};
}  // namespace

extern "C" {

// The gBGC likelihood engine on one element at one state.  bases: S rows of
// GG lower-case characters in tree leaf order; z, b: per node (b as 0/1);
// sc, sn, gb: conserved and accelerated selection and the GC bias.
// Outputs: logp [6][N][16] (classes null, cons, neut, null+B, cons+B,
// neut+B; 0 where not computed, as the reference's zero-initialised caches),
// col [GG] per-column log-likelihoods, counts [N][16] expected (child,
// parent) base counts (the root's in column 0), root, missing [N], and
// filtered (the conserved-species filter, bpp_c.hpp:297-311).

// One element through the gBGC model's three chains (M0, M2, M1 from one
// stream; main.cpp:383-412), with Eval2 and Output_init after each.  bases:
// S rows of GG lower-case characters in tree leaf order.
int oracle_gbgc_run_element(const pacc_model* m, const pacc_gbgc_opts* o, const uint8_t* bases, int32_t GG,
                            pacc_gbgc_result* r) {
    Elem E;
    std::set<int> upper;
    if (setup_element(m, bases, GG, o->gapchar, o->missing_thres, o->conserve_prop, E, upper)) {
        r->status = PACC_FILTERED;
        return PACC_FILTERED;
    }
    r->root = E.root;
    GChain C(m, o, E, upper);
    const int order[3] = {0, 2, 1};
    for (int q = 0; q < 3; q++) {
        const int resZ = order[q];
        if (!C.init(resZ) || !C.gibbs(resZ)) return PACC_EINVAL;
        r->max_loglik[resZ] = C.MaxLoglik;
        if (C.Max_Z.empty()) { C.Max_Z = C.Z; C.Max_B = C.B; }
        // the trace and tables before Eval2 and Output_init reorder anything
        C.output(resZ, r, resZ);
        const double ll = C.eval2(resZ);
        if (resZ == 0) r->loglik_null = ll;
        else if (resZ == 2) r->loglik_res = ll;
        else r->loglik_all = ll;
    }
    r->status = PACC_OK;
    return PACC_OK;
}

// Every element of a batch, elements spread over n_threads OpenMP threads
// like the reference's element loop (main.cpp:376-378, schedule guided).
int oracle_gbgc_run(const pacc_model* m, const pacc_gbgc_opts* o, const pacc_element_batch* b, pacc_gbgc_result* out,
                    int n_threads) {
    int bad = 0;
#pragma omp parallel for schedule(guided) num_threads(n_threads > 0 ? n_threads : 1) reduction(+ : bad)
    for (int i = 0; i < b->n_elements; i++) {
        out[i].element_no = b->element_no ? b->element_no[i] : i;
        const int st = oracle_gbgc_run_element(m, o, b->bases + b->offsets[i], b->lengths[i], &out[i]);
        if (st != PACC_OK && st != PACC_FILTERED) bad++;
    }
    return bad ? PACC_EINVAL : PACC_OK;
}

int oracle_gbgc_engine(const pacc_model* m, const uint8_t* bases, int32_t GG, int32_t gapchar, double missing_thres,
                       double conserve_prop, const int32_t* z, const int32_t* bflag, double sc, double sn, double gb,
                       double* logp, double* col, double* counts, int32_t* root_out, uint8_t* missing_out,
                       int32_t* filtered) {
    Elem E;
    std::set<int> upper;
    *filtered = setup_element(m, bases, GG, gapchar, missing_thres, conserve_prop, E, upper) ? 1 : 0;
    for (int s = 0; s < E.N; s++) missing_out[s] = (uint8_t)E.missing[s];
    if (*filtered) return PACC_FILTERED;
    const int S = E.S, N = E.N;
    // fixZ of the full model (bpp_c.cpp:144-150): the outgroup path is fixed
    std::vector<char> fixed(N, 0);
    for (int s : E.nodes)
        if (upper.count(s)) fixed[s] = 1;
    fixed[E.root] = 0;
    // rate matrices of the six classes (initMCMC, bpp_c.cpp:186-194) and
    // their per-branch log transition matrices (init_cache_TM)
    const double* Q0 = m->rate_matrix;
    M4 Qs[6];
    get_rate(Q0, 0, 0, Qs[0]);
    get_rate(Q0, sc, 0, Qs[1]);
    get_rate(Q0, sn, 0, Qs[2]);
    get_rate(Q0, 0, gb, Qs[3]);
    get_rate(Q0, sc, gb, Qs[4]);
    get_rate(Q0, sn, gb, Qs[5]);
    Eig eg[6];
    for (int k = 0; k < 6; k++)
        if (!eig_of(Qs[k], eg[k])) return PACC_EINVAL;
    std::memset(logp, 0, sizeof(double) * 6 * N * 16);
    for (size_t it = 0; it + 1 < E.nodes.size(); it++) {
        const int s = E.nodes[it];
        if (E.missing[s]) continue;
        for (int k = 0; k < 6; k++) {
            if ((k == 2 || k == 5) && fixed[s]) continue;
            M4 P;
            log_transition(eg[k], E.dist[s], P);
            for (int a = 0; a < 4; a++)
                for (int c = 0; c < 4; c++) logp[((size_t)k * N + s) * 16 + a * 4 + c] = P[a][c];
        }
    }
    // the branch's matrix (the switch on 2 Z + B of Update_Tg, bpp_c.cpp:494-517):
    // Z 0/1/2 without B -> null/cons/neut, with B -> null_B/cons_B/neut_B
    auto lp = [&](int s) -> const M4& {
        const int k = z[s] + (bflag[s] ? 3 : 0);
        return *reinterpret_cast<const M4*>(&logp[((size_t)k * N + s) * 16]);
    };
    double log_pi[4];
    for (int i = 0; i < 4; i++) log_pi[i] = std::log(m->pi[i]);
    std::memset(counts, 0, sizeof(double) * N * 16);
    std::vector<double> msg((size_t)N * 4);
    for (int g = 0; g < GG; g++) {
        std::vector<double>& L = E.lam[g];
        // pruning pass (bpp_c.cpp:480-515)
        for (int s : E.nodes) {
            if (s < S || E.missing[s]) continue;
            const int p[2] = {E.c0[s], E.c1[s]};
            for (int cc = 0; cc < 2; cc++) {
                const int chi = p[cc];
                if (E.missing[chi]) continue;
                log_multi(lp(chi), &L[(size_t)chi * 4], &msg[(size_t)chi * 4]);
                for (int j = 0; j < 4; j++) L[(size_t)s * 4 + j] += msg[(size_t)chi * 4 + j];
            }
        }
        for (int j = 0; j < 4; j++) L[(size_t)E.root * 4 + j] += log_pi[j];
        const double* lr = &L[(size_t)E.root * 4];
        col[g] = log_exp_sum4(lr);
        // sampling pass: expected counts (bpp_c.cpp:541-596)
        std::vector<double> ltp((size_t)N * 4, 0.0);
        double prob[4];
        {
            const double x = log_exp_sum4(lr);
            for (int j = 0; j < 4; j++) prob[j] = (x == INFINITY) ? 0.0 : std::exp(lr[j] - x);
        }
        for (int j = 0; j < 4; j++) {
            counts[(size_t)E.root * 16 + j * 4 + 0] += prob[j];
            ltp[(size_t)E.root * 4 + j] = std::log(prob[j]);
        }
        for (int it = (int)E.nodes.size() - 2; it >= 0; it--) {
            const int s = E.nodes[it];
            const int pa = E.parent[s];
            if (E.missing[s]) continue;
            const M4& T = lp(s);
            M4 tp;
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++)
                    tp[i][j] = T[i][j] + (ltp[(size_t)pa * 4 + j] - msg[(size_t)s * 4 + j]);
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) tp[i][j] += L[(size_t)s * 4 + i];
            // log_exp_rowsum (bpp.hpp:457-464): one max over the matrix
            const double mx = mat_max(tp);
            for (int i = 0; i < 4; i++) {
                double t = 0;
                for (int j = 0; j < 4; j++) t += std::exp(tp[i][j] - mx);
                ltp[(size_t)s * 4 + i] = std::log(t) + mx;
            }
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) counts[(size_t)s * 16 + i * 4 + j] += std::exp(tp[i][j]);
        }
    }
    *root_out = E.root;
    for (int s = 0; s < N; s++) missing_out[s] = (uint8_t)E.missing[s];
    return PACC_OK;
}

}  // extern "C"
