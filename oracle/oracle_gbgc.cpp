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

#include <cmath>
#include <cstring>
#include <set>
#include <vector>

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
int oracle_gbgc_engine(const pacc_model* m, const uint8_t* bases, int32_t GG, int32_t gapchar, double missing_thres,
                       double conserve_prop, const int32_t* z, const int32_t* bflag, double sc, double sn, double gb,
                       double* logp, double* col, double* counts, int32_t* root_out, uint8_t* missing_out,
                       int32_t* filtered) {
    Elem E;
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
    *filtered = ct > conserve_prop * m->n_conserve ? 1 : 0;
    if (*filtered) return PACC_FILTERED;
    // the outgroup path (getUppertree, bpp.cpp:454-476) and its collapse
    std::set<int> upper;
    for (int i = 0; i < m->n_outgroup; i++) {
        int p = m->outgroup[i];
        while (p != N - 1 && p >= 0 && p < N) { upper.insert(p); p = E.parent[p]; }
    }
    upper.insert(N - 1);
    subtree_missing(E, upper, N - 1, -1);
    E.parent[E.root] = N;
    postorder(E, E.root, E.nodes);
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
