// pacc_host.cpp — host side of the C ABI declared in include/pacc.h.
//
// Owns the context (model constants, device buffers), the per-element
// preprocessing that PhyloAcc-ST does in the BPP_C constructor
// (src/PhyloAcc-ST/bpp_c.hpp:143-476: column encoding, optional column
// trimming, missing taxa, pruning of the outgroup path, node orders), the
// packing of elements into one device blob, the kernel launches and the
// collection of results.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <array>
#include <deque>
#include <map>
#include <unordered_map>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pacc.h"
#include "eigen4.h"
#include "pacc_dev.h"

namespace pacc {

cudaError_t set_model(const DevModel& m, cudaStream_t st);
size_t smem_bytes(int N, int BT, int prec, int D);
int chain_occupancy(int prec, int variant, int BT, size_t smem);
int chain_variants(int prec);
int chain_variant_max_threads(int prec, int v);
size_t ws_bytes(int n_int, int GGp, int T, int mcmc, int N, int prec);
size_t topo_bytes(int N);
cudaError_t launch_chain(const ChainParams& p, int grid, int BT, size_t smem, int prec, int variant, cudaStream_t st);
cudaError_t launch_loglik(const ChainParams& p, const int32_t* z, double c_rate, double n_rate, double* out, int BT,
                          size_t smem, int prec, cudaStream_t st);
cudaError_t launch_pmatrix(int n, const double* d, const double* r, double* out, cudaStream_t st);
cudaError_t launch_stream(uint32_t seed, uint64_t w0, int n, uint32_t* out, cudaStream_t st);
cudaError_t launch_fma_probe(int prec, int grid, int BT, int iters, void* out, cudaStream_t st);
cudaError_t set_model_batch(const DevModel& m, cudaStream_t st);
size_t batch_warp_smem(int N, int NI, int S, int D, int prec, int C);
size_t batch_slot_bytes(int N, int T);
size_t batch_grp_bytes(int mcmc, int NI, int prec, int GGuP, int N);
cudaError_t noalloc_scratch_address(double** p);
bool batch_supports(int prec, int C);
int batch_occupancy(int prec, int C, int warps, size_t smem);
cudaError_t launch_init_slots(void* slots, const int32_t* elem, int n, cudaStream_t st);
cudaError_t launch_batch(const void* params, int grid, int warps, size_t smem, int prec, int C, cudaStream_t st);
cudaError_t launch_gbgc(const GbgcParams& p, int prec, cudaStream_t st);
size_t gbgc_chain_smem(int N, int prec);
int gbgc_chain_threads();
int gbgc_chain_warps();
int gbgc_chain_occupancy(int prec, int regs, size_t smem);
cudaError_t launch_gbgc_chain(const GbgcChainParams& p, int grid, size_t smem, int prec, int regs, cudaStream_t st);

// ---------------------------------------------------------------------------
// model (BPP, bpp.hpp:173-404)
// ---------------------------------------------------------------------------
struct HostModel {
    int S = 0, N = 0;
    std::vector<int> ch0, ch1, parent;
    std::vector<double> dist;
    std::vector<int> conserve, outgroup;
    std::vector<char> upper, upper_conserve;  // [N]
    double rate[16], pi[4];                   // RATE_MAT (row-major, i -> j) and BACKGROUND
    DevModel dm;
};

// One preprocessed element.
struct HostElem {
    int64_t no = 0;
    int filtered = 0;
    int GG = 0, GGp = 0, root = 0, n_nodes = 0, n_int = 0, n_hlev = 0, n_dlev = 0, tg_draws = 0;
    std::vector<uint8_t> codes;    // [S][GGp]
    std::vector<uint8_t> codes_t;  // [GGp][SP] column-major copy for 128-bit per-column loads
    int GGu = 0;                   // distinct site patterns
    std::vector<uint8_t> pcodes_t; // [GGu rounded up to 32][SP] the patterns in first-occurrence order
    std::vector<int32_t> pw;       // [GGu] columns per pattern
    std::vector<int32_t> pattern_of;  // [GG] pattern of each column
    std::vector<int8_t> tg0;       // [n_int][GGp]
    std::vector<int32_t> prefix;   // [GG+1]
    std::vector<int16_t> topo;     // TopoLayout
    std::vector<double> dist2;     // [N]
    std::vector<int8_t> tg_full;   // [GG][N] (debug encode only)
    std::vector<uint8_t> missing;  // [N]
    std::vector<int> sord, sflag;  // stack order of internal nodes, pop-order flags
    int stack_depth = 0;
    std::vector<int8_t> start_z;   // SAMPLE_HYPER start state ([N], empty: the first chain's start)
    std::vector<double> start_rates;  // [5] n, c, g, l, l2 (empty: the INIT_* values)
};

static inline uint8_t encode_char(uint8_t ch, char gapchar) {
    // bpp_c.hpp:220-261
    switch ((char)ch) {
        case 'a': return CODE_A;
        case 'c': return CODE_C;
        case 'g': return CODE_G;
        case 't': return CODE_T;
        case 'r': return CODE_R;
        case 'y': return CODE_Y;
        case 'k': return CODE_K;
        case 'm': return CODE_M;
        case 's': return CODE_S;
        case 'w': return CODE_W;
        default: return ((char)ch == gapchar) ? CODE_GAP : CODE_OTHER;
    }
}

static inline int code_tg(uint8_t c) { return c < 4 ? c : (c == CODE_GAP ? 4 : (c == CODE_OTHER ? 5 : -1)); }

// Site patterns: the distinct columns (all taxa's codes equal) in order of
// first occurrence, with the number of columns of each.  A column's
// likelihood depends only on its codes, so the likelihood passes run once per
// pattern and weight it; the internal-base draws still run per column.
static void compress_patterns(HostElem& E, int SP) {
    const int GG = E.GG;
    size_t cap = 16;
    while (cap < (size_t)GG * 2) cap <<= 1;
    std::vector<int32_t> slot(cap, -1);  // open addressing: pattern id
    std::vector<int32_t> first;          // first column of each pattern
    E.pattern_of.assign(GG, 0);
    E.pw.clear();
    for (int g = 0; g < GG; g++) {
        const uint8_t* col = &E.codes_t[(size_t)g * SP];
        uint64_t h = 1469598103934665603ull;
        for (int s = 0; s < SP; s++) h = (h ^ col[s]) * 1099511628211ull;
        size_t i = (size_t)(h ^ (h >> 29)) & (cap - 1);
        int pid = -1;
        while (slot[i] >= 0) {
            const int q = slot[i];
            if (std::memcmp(&E.codes_t[(size_t)first[q] * SP], col, SP) == 0) { pid = q; break; }
            i = (i + 1) & (cap - 1);
        }
        if (pid < 0) {
            pid = (int)first.size();
            first.push_back(g);
            E.pw.push_back(0);
            slot[i] = pid;
        }
        E.pattern_of[g] = pid;
        E.pw[pid]++;
    }
    E.GGu = (int)first.size();
    const int GGuP = (E.GGu + 31) & ~31;
    E.pcodes_t.assign((size_t)std::max(GGuP, 32) * SP, CODE_GAP);
    for (int p = 0; p < E.GGu; p++)
        std::memcpy(&E.pcodes_t[(size_t)p * SP], &E.codes_t[(size_t)first[p] * SP], SP);
}

// Collapse the missing branches of the nodes marked in up, moving the root
// down where the root itself loses a child (getSubtree_missing,
// bpp_c.cpp:64-113; the same walk in PhyloAcc-ST-GBGC, bpp_c.cpp:53-111).
static void collapse_missing_path(int S, const std::vector<char>& up, std::vector<int>& c2a, std::vector<int>& c2b,
                                  std::vector<int>& par, std::vector<double>& d2, const std::vector<char>& missing,
                                  int& root) {
    struct Walker {
        int S;
        const std::vector<char>& up;
        std::vector<int>&c2a, &c2b, &par;
        std::vector<double>& d2;
        const std::vector<char>& missing;
        int& root;
        void walk(int ss, int child) {
            if (!up[ss] || ss < S) return;
            int s = ss;
            while (up[s] && s >= S) {
                int p0 = c2a[s], p1 = c2b[s];
                int keep;
                if (missing[p0] && !missing[p1]) { keep = p1; par[p0] = -1; }
                else if (!missing[p0] && missing[p1]) { keep = p0; par[p1] = -1; }
                else {
                    walk(p0, 0);
                    walk(p1, 1);
                    return;
                }
                d2[keep] += d2[s];
                if (s == root) root = keep;
                else {
                    (child == 0 ? c2a : c2b)[par[ss]] = keep;
                    par[keep] = par[ss];
                }
                s = keep;
            }
        }
    } wk{S, up, c2a, c2b, par, d2, missing, root};
    wk.walk(root, -1);
}

// Postorder of the tree below root, first children first (bpp_c.cpp:44-60).
static std::vector<int> postorder_nodes(int root, const std::vector<int>& c2a, const std::vector<int>& c2b) {
    std::vector<int> nodes;
    nodes.reserve(c2a.size());
    std::vector<std::pair<int, int>> st;
    st.push_back({root, 0});
    while (!st.empty()) {
        auto& t = st.back();
        int j = t.first;
        if (t.second == 0) {
            t.second = 1;
            if (c2a[j] != -1) { st.push_back({c2a[j], 0}); continue; }
        }
        if (t.second == 1) {
            t.second = 2;
            if (c2b[j] != -1) { st.push_back({c2b[j], 0}); continue; }
        }
        nodes.push_back(j);
        st.pop_back();
    }
    return nodes;
}

// One element of the PhyloAcc-ST-GBGC model, preprocessed for its
// likelihood engine (BPP_C ctor of that model, src/PhyloAcc-ST-GBGC/SRC/
// bpp_c.hpp:153-379): allowed-base masks per leaf and column, missing taxa,
// the conserved-species filter, and the tree with the missing outgroup path
// collapsed (getSubtree_missing, bpp_c.cpp:53-111).
struct GbgcElem {
    int GG = 0, GGp = 0, root = 0, filtered = 0;
    std::vector<uint8_t> masks;          // [S][GGp]
    std::vector<char> missing, fixed;    // [N]
    std::vector<int> c2a, c2b, par;      // [N] after the collapse
    std::vector<double> d2;              // [N]
    std::vector<int> nodes;              // postorder from root
};

// bit i: base i (A, C, G, T) allowed (bpp_c.hpp:203-251 of the gBGC model);
// '-', 'n', the gap character and anything else allow all four
static inline uint8_t gbgc_mask(uint8_t ch) {
    switch ((char)ch) {
        case 'a': return 1;
        case 'c': return 2;
        case 'g': return 4;
        case 't': return 8;
        case 'r': return 1 | 4;
        case 'y': return 2 | 8;
        case 'k': return 4 | 8;
        case 'm': return 1 | 2;
        case 's': return 2 | 4;
        case 'w': return 1 | 8;
        default: return 15;
    }
}

static void gbgc_prepare(const HostModel& M, const uint8_t* bases, int GG, char gapchar, double missing_thres,
                         double conserve_prop, GbgcElem& E) {
    const int S = M.S, N = M.N;
    E.GG = GG;
    E.GGp = (GG + 31) & ~31;
    E.masks.assign((size_t)S * E.GGp, 15);
    std::vector<int> num_missing(S, 0);
    for (int s = 0; s < S; s++)
        for (int g = 0; g < GG; g++) {
            const uint8_t ch = bases[(size_t)s * GG + g];
            if ((char)ch == gapchar) num_missing[s]++;
            E.masks[(size_t)s * E.GGp + g] = gbgc_mask(ch);
        }
    E.missing.assign(N, 0);
    for (int s = S; s < N; s++) {
        const int p[2] = {M.ch0[s], M.ch1[s]};
        for (int q = 0; q < 2; q++)
            if (p[q] < S && num_missing[p[q]] > missing_thres * GG) E.missing[p[q]] = 1;
        if (E.missing[p[0]] && E.missing[p[1]]) E.missing[s] = 1;
    }
    int ct = 0;
    for (int cidx : M.conserve) if (cidx >= 0 && cidx < N && E.missing[cidx]) ct++;
    if (ct > conserve_prop * (double)M.conserve.size()) { E.filtered = 1; return; }
    E.c2a = M.ch0; E.c2b = M.ch1; E.par = M.parent; E.d2 = M.dist;
    E.root = N - 1;
    collapse_missing_path(S, M.upper, E.c2a, E.c2b, E.par, E.d2, E.missing, E.root);
    E.par[E.root] = N;
    E.nodes = postorder_nodes(E.root, E.c2a, E.c2b);
    // the outgroup path has no accelerated class (fixZ, bpp_c.cpp:144-150)
    E.fixed.assign(N, 0);
    for (int s : E.nodes) if (M.upper[s] && s != E.root) E.fixed[s] = 1;
}


// ---------------------------------------------------------------------------
// The gBGC chain (PhyloAcc-ST-GBGC): element blobs for the chain kernel, and
// Eval2 / Output_init on the host from the traces the kernel writes.
// ---------------------------------------------------------------------------

// Element blob of the chain kernel: the collapsed tree, its levels and the
// leaf columns (GbgcElemHdr gives the offsets).
static void gbgc_blob(const HostModel& M, const GbgcElem& E, GbgcElemHdr& H, std::vector<uint8_t>& out) {
    const int S = M.S, N = M.N;
    const int nn = (int)E.nodes.size();
    std::vector<int> height(N, 0), depth(N, 0), pidx(N, -1);
    for (int k = 0; k < nn; k++) pidx[E.nodes[k]] = k;
    int H_max = 0;
    for (int s : E.nodes)
        if (s >= S) {
            height[s] = 1 + std::max(height[E.c2a[s]], height[E.c2b[s]]);
            H_max = std::max(H_max, height[s]);
        }
    int D_max = 0;
    for (int k = nn - 1; k >= 0; k--) {
        const int s = E.nodes[k];
        depth[s] = (s == E.root) ? 0 : depth[E.par[s]] + 1;
        D_max = std::max(D_max, depth[s]);
    }
    std::vector<int16_t> hstart, hnodes, dstart, dnodes;
    for (int h = 1; h <= H_max; h++) {
        hstart.push_back((int16_t)hnodes.size());
        for (int s : E.nodes)
            if (s >= S && height[s] == h) hnodes.push_back((int16_t)s);
    }
    hstart.push_back((int16_t)hnodes.size());
    for (int d = 1; d <= D_max; d++) {
        dstart.push_back((int16_t)dnodes.size());
        for (int k = nn - 1; k >= 0; k--)
            if (E.nodes[k] != E.root && depth[E.nodes[k]] == d) dnodes.push_back((int16_t)E.nodes[k]);
    }
    dstart.push_back((int16_t)dnodes.size());
    out.clear();
    auto put = [&](const void* src, size_t bytes, size_t align) -> int32_t {
        while (out.size() % align) out.push_back(0);
        const int32_t o = (int32_t)out.size();
        out.insert(out.end(), (const uint8_t*)src, (const uint8_t*)src + bytes);
        return o;
    };
    std::vector<int16_t> nodes(N, 0), c0(N), c1(N), par(N), irank(N), pi16(N);
    std::vector<uint8_t> flags(N);
    for (int k = 0; k < nn; k++) nodes[k] = (int16_t)E.nodes[k];
    for (int s = 0; s < N; s++) {
        c0[s] = (int16_t)E.c2a[s];
        c1[s] = (int16_t)E.c2b[s];
        par[s] = (int16_t)std::min(E.par[s], N);
        irank[s] = (int16_t)(s >= S ? s - S : -1);
        pi16[s] = (int16_t)pidx[s];
        flags[s] = (uint8_t)((E.missing[s] ? GBGC_MISSING : 0) | (M.upper[s] ? GBGC_UPPER : 0));
    }
    H.S = S; H.N = N; H.GG = E.GG; H.GGp = E.GGp; H.root = E.root; H.n_nodes = nn; H.n_int = S - 1;
    H.n_hlev = H_max; H.n_dlev = D_max;
    H.o_nodes = put(nodes.data(), 2 * N, 16);
    H.o_c0 = put(c0.data(), 2 * N, 2);
    H.o_c1 = put(c1.data(), 2 * N, 2);
    H.o_par = put(par.data(), 2 * N, 2);
    H.o_irank = put(irank.data(), 2 * N, 2);
    H.o_pidx = put(pi16.data(), 2 * N, 2);
    H.o_flags = put(flags.data(), N, 1);
    H.o_dist = put(E.d2.data(), 8 * (size_t)N, 8);
    H.o_hlev = put(hstart.data(), 2 * hstart.size(), 2);
    hnodes.resize((size_t)std::max(S - 1, (int)hnodes.size()), 0);   // the kernel copies S - 1 entries
    H.o_hnodes = put(hnodes.data(), 2 * hnodes.size(), 2);
    H.o_dlev = put(dstart.data(), 2 * dstart.size(), 2);
    H.o_dnodes = put(dnodes.data(), 2 * dnodes.size(), 2);
    // the branches that are not missing, by length (ties by id)
    std::vector<int16_t> blen;
    for (int k = 0; k + 1 < nn; k++)
        if (!E.missing[E.nodes[k]]) blen.push_back((int16_t)E.nodes[k]);
    std::stable_sort(blen.begin(), blen.end(), [&](int16_t a, int16_t b2) {
        return E.d2[a] < E.d2[b2] || (E.d2[a] == E.d2[b2] && a < b2);
    });
    H.n_blen = (int32_t)blen.size();
    H.o_blen = put(blen.data(), 2 * blen.size() + 2, 2);
    H.o_masks = put(E.masks.data(), E.masks.size(), 16);
    while (out.size() % 16) out.push_back(0);
    H.blob_off = 0;
}

// Eval2 (bpp_c2.cpp:29-286) of one model from its trace: the marginal
// log-likelihood.  trd: [4][T] full loglik, n, c, gBC; tz / tb: Z and B of
// sample i at tz[i * stride + s] / tb[i * stride + s].
static double gbgc_eval2(int resZ, int T, int burn, int mcmc, int N, const std::vector<int>& nodes,
                         const std::vector<char>& missing, const double* trd, const int8_t* tz, const int8_t* tb,
                         size_t stride, const int8_t* maxz, double max_loglik) {
    const double* tr_full = trd;
    const double* tr_n = trd + T;
    const double* tr_c = trd + 2 * T;
    const double* tr_gb = trd + 3 * T;
    std::vector<int> uncertain;
    for (int s = 0; s < N; s++) {
        int c = 0;
        for (int i = burn; i < T; i++)
            if (tz[(size_t)i * stride + s] == maxz[s]) c++;
        if (c < mcmc) uncertain.push_back(s);
    }
    const int d = 2 + (resZ != 0 ? 1 : 0);
    auto zkey = [&](const int8_t* z) {
        std::string k(uncertain.size(), '\0');
        for (size_t u = 0; u < uncertain.size(); u++) k[u] = (char)z[uncertain[u]];
        return k;
    };
    std::unordered_map<std::string, int> cfg;
    cfg.emplace(zkey(maxz), 0);
    std::vector<int> nZ(1, 0);
    std::vector<std::unordered_map<std::string, int>> zbIndex(1);
    std::vector<std::vector<int>> nZB(1);
    std::vector<std::vector<double>> means(1, std::vector<double>(d, 0.0)), var(1, std::vector<double>(d * d, 0.0));
    std::vector<double> sumf(1, 0.0);
    std::string bkey;
    for (int i = T - 1; i >= burn; i--) {
        const int8_t* z = tz + (size_t)i * stride;
        const int8_t* b = tb + (size_t)i * stride;
        auto ins = cfg.emplace(zkey(z), (int)nZ.size());
        const int j = ins.first->second;
        if (ins.second) {
            nZ.push_back(0);
            zbIndex.emplace_back();
            nZB.emplace_back();
            means.emplace_back(d, 0.0);
            var.emplace_back(d * d, 0.0);
            sumf.push_back(0.0);
        }
        nZ[j]++;
        // getShifts (bpp_c2.cpp:14-27): the element's branches with B = 1
        bkey.assign((size_t)N, '\0');
        for (int s : nodes)
            if (!missing[s] && b[s]) bkey[s] = 1;
        auto kb = zbIndex[j].emplace(bkey, (int)nZB[j].size());
        if (kb.second) nZB[j].push_back(0);
        nZB[j][kb.first->second]++;
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
    auto log_det = [&](std::vector<double> u, double& val, double& sign) {   // LU, partial pivoting
        sign = 1.0;
        val = 0.0;
        for (int k = 0; k < d; k++) {
            int pv = k;
            for (int i = k + 1; i < d; i++)
                if (std::fabs(u[k * d + i]) > std::fabs(u[k * d + pv])) pv = i;
            if (pv != k) {
                for (int j = 0; j < d; j++) std::swap(u[j * d + k], u[j * d + pv]);
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
    for (size_t i = 0; i < nZ.size(); i++) {
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
        for (size_t i = 0; i < nZ.size(); i++) {
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
    if (resZ == 1 && eff == 0) return max_loglik;
    return VB / eff + std::log((double)eff) + (double)d / 2 * std::log(2 * M_PI);
}

// Per-element preprocessing (BPP_C ctor, bpp_c.hpp:143-476).  Returns false
// only on invalid input; filtered elements return true with E.filtered = 1.
static bool preprocess(const HostModel& M, const pacc_opts& o, const uint8_t* bases, int len, HostElem& E,
                       bool keep_full) {
    const int S = M.S, N = M.N;
    E.GG = len;
    if (len < o.min_len) { E.filtered = 1; return true; }
    // encode (species rows, tree leaf order)
    std::vector<uint8_t> code((size_t)S * len);
    const char gapchar = (char)o.gapchar;
    for (int s = 0; s < S; s++)
        for (int g = 0; g < len; g++) code[(size_t)s * len + g] = encode_char(bases[(size_t)s * len + g], gapchar);
    // optional column trimming (bpp_c.hpp:267-301)
    std::vector<int> cols;
    cols.reserve(len);
    if (o.trim_gap_percent < 1) {
        int nmis = 0;
        for (int g = 0; g < len; g++) {
            int mis = 0;
            for (int s = 0; s < S; s++) if (code_tg(code[(size_t)s * len + g]) >= 4) mis++;
            if (mis > S * o.trim_gap_percent) nmis++;
            else cols.push_back(g);
        }
        if (len - nmis < o.min_len) { E.filtered = 1; return true; }
    } else {
        for (int g = 0; g < len; g++) cols.push_back(g);
    }
    const int GG = (int)cols.size();
    E.GG = GG;
    E.GGp = (GG + 31) & ~31;
    const int GGp = E.GGp;
    E.codes.assign((size_t)S * GGp, CODE_GAP);
    for (int s = 0; s < S; s++)
        for (int i = 0; i < GG; i++) E.codes[(size_t)s * GGp + i] = code[(size_t)s * len + cols[i]];
    const int SP = (S + 15) & ~15;
    E.codes_t.assign((size_t)GGp * SP, CODE_GAP);
    for (int i = 0; i < GG; i++)
        for (int s = 0; s < S; s++) E.codes_t[(size_t)i * SP + s] = E.codes[(size_t)s * GGp + i];
    compress_patterns(E, SP);
    // gap counts and missing flags (bpp_c.hpp:303-351)
    std::vector<int> num_missing(S, 0);
    for (int s = 0; s < S; s++)
        for (int i = 0; i < GG; i++) if (E.codes[(size_t)s * GGp + i] == CODE_GAP) num_missing[s]++;
    std::vector<int> c2a = M.ch0, c2b = M.ch1, par = M.parent;
    std::vector<double> d2 = M.dist;
    std::vector<char> missing(N, 0);
    for (int s = S; s < N; s++) {
        int p[2] = {c2a[s], c2b[s]};
        for (int q = 0; q < 2; q++)
            if (p[q] < S && num_missing[p[q]] > o.gap_prop * GG) missing[p[q]] = 1;
        if (missing[p[0]] && missing[p[1]]) missing[s] = 1;
    }
    int ct = 0;
    for (int cidx : M.conserve) if (cidx >= 0 && cidx < N && missing[cidx]) ct++;
    if (ct > o.conserve_prop * (double)M.conserve.size()) { E.filtered = 1; return true; }
    // collapse missing branches on the outgroup path, or everywhere with PRUNE_TREE
    // (getSubtree_missing, bpp_c.cpp:64-113)
    int root = N - 1;
    std::vector<char> up(N, 0);
    for (int s = 0; s < N; s++) up[s] = o.prune_tree ? 1 : M.upper[s];
    collapse_missing_path(S, up, c2a, c2b, par, d2, missing, root);
    par[root] = N;
    const std::vector<int> nodes = postorder_nodes(root, c2a, c2b);
    std::vector<int> internal;
    for (int s : nodes) if (s >= S) internal.push_back(s);
    if (internal.empty()) { E.filtered = 2; return true; }  // the whole tree collapsed to one leaf
    const int n_int = (int)internal.size();
    std::vector<int> irank(N, -1), pos(N, -1);
    for (int i = 0; i < n_int; i++) irank[internal[i]] = i;
    for (int i = 0; i < (int)nodes.size(); i++) pos[nodes[i]] = i;
    // internal Tg = K where both children are >= K (bpp_c.hpp:417-428)
    E.tg0.assign((size_t)n_int * GGp, 4);
    auto tg_at = [&](int s, int g) -> int {
        if (s < S) return code_tg(E.codes[(size_t)s * GGp + g]);
        return E.tg0[(size_t)irank[s] * GGp + g];
    };
    for (int i = 0; i < n_int; i++) {
        int s = internal[i];
        for (int g = 0; g < GG; g++)
            E.tg0[(size_t)i * GGp + g] = (tg_at(c2a[s], g) >= 4 && tg_at(c2b[s], g) >= 4) ? 4 : -1;
    }
    // stream words of one internal-base pass: per column the root and every
    // eligible internal node (bpp_c.cpp:674-732)
    E.prefix.assign(GG + 1, 0);
    for (int g = 0; g < GG; g++) {
        int cnt = 1;
        for (int i = 0; i + 1 < n_int; i++) {
            int s = internal[i];
            if (!missing[s] && E.tg0[(size_t)i * GGp + g] < 4) cnt++;
        }
        E.prefix[g + 1] = E.prefix[g] + cnt;
    }
    E.tg_draws = E.prefix[GG];
    // levels: heights of internal nodes for the upward filter, depths for sampling
    std::vector<int> height(N, 0), depth(N, 0);
    for (int s : nodes)
        if (s >= S) height[s] = 1 + std::max(height[c2a[s]], height[c2b[s]]);
    for (int i = (int)nodes.size() - 1; i >= 0; i--) {
        int s = nodes[i];
        depth[s] = (s == root) ? 0 : depth[par[s]] + 1;
    }
    TopoLayout TL = TopoLayout::make(N);
    E.topo.assign(TL.total, 0);
    int16_t* t = E.topo.data();
    for (int i = 0; i < N; i++) {
        t[TL.nodes + i] = (int16_t)(i < (int)nodes.size() ? nodes[i] : -1);
        t[TL.internal + i] = (int16_t)(i < n_int ? internal[i] : -1);
        t[TL.c2a + i] = (int16_t)c2a[i];
        t[TL.c2b + i] = (int16_t)c2b[i];
        t[TL.par + i] = (int16_t)par[i];
        t[TL.irank + i] = (int16_t)irank[i];
        t[TL.pos + i] = (int16_t)pos[i];
        t[TL.missing + i] = (int16_t)missing[i];
        t[TL.upc + i] = (int16_t)(M.upper[i] ? 1 : 0);
        t[TL.upcc + i] = (int16_t)(M.upper_conserve[i] ? 1 : 0);
    }
    int maxh = 0, maxd = 0;
    for (int s : nodes) { if (s >= S) maxh = std::max(maxh, height[s]); maxd = std::max(maxd, depth[s]); }
    {
        int k = 0;
        for (int h = 1; h <= maxh; h++) {
            t[TL.hlev_start + h - 1] = (int16_t)k;
            for (int s : nodes) if (s >= S && height[s] == h) t[TL.hlev_nodes + k++] = (int16_t)s;
        }
        t[TL.hlev_start + maxh] = (int16_t)k;
        E.n_hlev = maxh;
        k = 0;
        for (int d = 1; d <= maxd; d++) {
            t[TL.dlev_start + d - 1] = (int16_t)k;
            for (int s : nodes) if (depth[s] == d) t[TL.dlev_nodes + k++] = (int16_t)s;
        }
        t[TL.dlev_start + maxd] = (int16_t)k;
        E.n_dlev = maxd;
    }
    // stack order for the batched kernel: a postorder that visits the child
    // subtree needing more pending partials first (Sethi-Ullman), so that at
    // most E.stack_depth partials are pending at once
    {
        std::vector<int> need(N, 0);
        for (int s : nodes) {
            if (s < S) continue;
            int a = c2a[s], b = c2b[s];
            int na = a >= S ? need[a] : 0, nb = b >= S ? need[b] : 0;
            if (a < S && b < S) need[s] = 1;
            else if (a < S) need[s] = std::max(nb, 1);
            else if (b < S) need[s] = std::max(na, 1);
            else need[s] = std::max(std::max(na, nb), 1 + std::min(na, nb));
        }
        E.stack_depth = need[root];
        std::vector<int> sord;
        std::vector<int> sflag(N, 0);
        std::vector<std::pair<int, int>> st;  // (node, state)
        st.push_back({root, 0});
        while (!st.empty()) {
            auto cur = st.back();
            st.pop_back();
            int s = cur.first;
            if (s < S) continue;
            if (cur.second == 1) { sord.push_back(s); continue; }
            int a = c2a[s], b = c2b[s];
            bool a_int = a >= S, b_int = b >= S;
            int first = a, second = b;
            if (a_int && b_int && need[b] > need[a]) { first = b; second = a; sflag[s] = 1; }
            st.push_back({s, 1});
            st.push_back({second, 0});
            st.push_back({first, 0});
        }
        E.sord = sord;
        E.sflag = sflag;
    }
    for (int i = 0; i < N; i++) {
        t[TL.sord + i] = (int16_t)(i < (int)E.sord.size() ? E.sord[i] : -1);
        t[TL.sflag + i] = (int16_t)E.sflag[i];
    }
    E.dist2 = d2;
    E.root = root;
    E.n_nodes = (int)nodes.size();
    E.n_int = n_int;
    E.missing.assign(missing.begin(), missing.end());
    if (keep_full) {
        E.tg_full.assign((size_t)GG * N, -1);
        for (int g = 0; g < GG; g++) {
            for (int s = 0; s < S; s++) E.tg_full[(size_t)g * N + s] = (int8_t)code_tg(E.codes[(size_t)s * GGp + g]);
            for (int i = 0; i < n_int; i++) E.tg_full[(size_t)g * N + internal[i]] = E.tg0[(size_t)i * GGp + g];
        }
    }
    return true;
}

}  // namespace pacc

using namespace pacc;

// Serving state: chain slots resident on the device, admitted from a host
// queue as slots free up, advanced by a CUDA-graph-captured sweep step.
struct Server {
    bool ready = false;
    int n_slots = 0, warps = 4, grid = 0, prec = 1, C = 1, D = 1, n_int_max = 1, GG_cap = 0, SP = 16;
    size_t smem = 0, slot_b = 0, grp_b = 0, blob_b = 0, tb = 0, o_prefix = 0, o_codes = 0, o_pcodes = 0, o_pw = 0,
           o_pof = 0;
    char* h_stage = nullptr;   // pinned staging of admitted elements
    size_t h_stage_cap = 0;
    bool inflight = false;     // a sweep was launched and not yet retired
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    char* dev = nullptr;
    ElemHeader* d_hdr = nullptr;
    char* d_blob = nullptr;
    SlotState* d_slots = nullptr;
    char* d_slotws = nullptr;
    char* d_grp = nullptr;
    DevResult* d_res = nullptr;
    int32_t* d_mz = nullptr;
    double* d_pz = nullptr;
    DevCounters* d_cnt = nullptr;
    double* d_trd = nullptr;
    int8_t* d_trz = nullptr;
    int TI = 0;
    int* d_ctr = nullptr;       // [0] n_done, [32] next_slot
    int* d_done = nullptr;
    int* h_done = nullptr;      // pinned: [0] count, [1..] slots
    BatchParams p;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    std::vector<int> free_slots;
    std::vector<int64_t> slot_no;
    std::vector<double> slot_t0;
    std::deque<std::pair<HostElem, double>> queue;
    int resident = 0;
    long long steps = 0;
    double kernel_ms = 0;
};

// Serving with the CTA-per-chain kernel: one persistent launch whose CTAs
// take element slots from a queue in host-mapped memory that the host appends
// to while the kernel runs, so chains of new requests start as soon as a CTA
// is free (continuous batching without relaunches).  A CTA that finds no work
// for a while returns; the host launches again when work arrives.
struct StreamServer {
    bool ready = false;
    int n_slots = 0, grid = 0, BT = 128, variant = 0, prec = 0, GG_cap = 0, GGp_cap = 0, n_int_cap = 0, TI = 0;
    size_t smem = 0, ws1 = 0, blob_b = 0, o_tg = 0, o_prefix = 0, o_topo = 0;
    char* dev = nullptr;
    ElemHeader* d_hdr = nullptr;
    char* d_blob = nullptr;
    DevResult* d_res = nullptr;
    int32_t* d_mz = nullptr;
    double* d_pz = nullptr;
    double* d_trd = nullptr;
    int8_t* d_trz = nullptr;
    DevCounters* d_cnt = nullptr;
    int* d_head = nullptr;
    char* d_ws = nullptr;
    int* h_map = nullptr;           // host-mapped: [0] tail, [1] stop, [64, 64+n) slot ring, [64+n, 64+2n) done flags
    volatile int* h_tail = nullptr;
    volatile int* h_stop = nullptr;
    bool stopping = false;          // the idle blocks were asked to return
    volatile int* h_qslot = nullptr;
    volatile int* h_done = nullptr;
    cudaStream_t copy = nullptr;    // admission and result copies, beside the running kernel
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool running = false;
    // pinned staging, allocated once at setup: cudaFreeHost / cudaMallocHost
    // synchronise the device, which would wait for the persistent launch
    char* h_stage = nullptr;
    size_t h_stage_cap = 0;
    char* h_out = nullptr;          // result staging for out_chunk slots
    int out_chunk = 0;
    ChainParams p;
    std::vector<int> free_slots;
    std::vector<char> busy;
    std::vector<int64_t> slot_no;
    std::vector<double> slot_t0;
    std::deque<std::pair<HostElem, double>> queue;
    int resident = 0, tail = 0;
    long long launches = 0;
    double kernel_ms = 0;
    DevCounters carry{};            // device counters of earlier set-ups of this context
};


// The gBGC model's serving state: a persistent chain kernel fed from a host
// queue (slots of element blob + outputs on the device, a mapped ring of
// queue positions and per-slot done flags); everything is allocated once at
// set-up, because allocations synchronise the device and would wait for the
// persistent launch.
struct GbgcServer {
    bool ready = false, running = false;
    int ns = 0, grid = 0, prec = 0, regs = 96, N = 0, T = 0, GGp_cap = 0;
    size_t smem = 0, blob_cap = 0, out_b = 0;
    pacc_gbgc_opts g;
    std::vector<int32_t> target;
    char* dev = nullptr;
    GbgcElemHdr* d_hdr = nullptr;
    char* d_blob = nullptr;
    char* d_out = nullptr;          // per slot: tr_d, tr_zb, max_zb, max_ll, status
    int* h_map = nullptr;           // host-mapped: [0] tail, [1] stop, [64, 64+ns) slot ring, [64+ns, 64+2ns) done
    volatile int *h_tail = nullptr, *h_stop = nullptr, *h_qslot = nullptr, *h_done = nullptr;
    char* h_stage = nullptr;        // pinned admission staging
    size_t h_stage_cap = 0;
    char* h_out = nullptr;          // pinned result staging, out_chunk slots
    int out_chunk = 0;
    cudaStream_t copy = nullptr;
    cudaEvent_t ev_done = nullptr, ev0 = nullptr;
    GbgcChainParams p;
    std::vector<int> free_slots;
    std::vector<char> busy;
    std::vector<int64_t> slot_no;
    std::vector<double> slot_t0;
    std::vector<GbgcElem> slot_elem;
    struct Pending {
        GbgcElem E;
        GbgcElemHdr H;
        std::vector<uint8_t> blob;
        int64_t no;
        double t0;
        int filtered;
    };
    std::deque<Pending> queue;
    struct Done {
        pacc_gbgc_result r;
        std::vector<int32_t> max_z;
        std::vector<int8_t> max_b;
        std::vector<double> post_b, post_z;
    };
    std::deque<Done> done;
    int tail = 0, resident = 0;
    long long launches = 0;
    double kernel_ms = 0;
    unsigned long long* d_idle = nullptr;
};

struct pacc_ctx {
    HostModel M;
    pacc_opts o;
    std::string err;
    int device = 0;
    int n_sm = 0;
    int stack_cap = 1;       // pending partials of the CTA kernel's prune (the full tree's stack order)
    // launch shape of the CTA-per-chain kernel (chosen at the first launch)
    bool shape_ready = false;
    int shape_variant = 0, shape_bt = 128, shape_per_sm = 0;
    double shape_trial_ms = 0;
    bool gpu_ok = false;
    cudaStream_t stream = nullptr;
    cudaStream_t aux = nullptr;   // the allocation-free entry point's own stream (beside a serving launch)
    // pending and finished work
    std::vector<HostElem> pending;
    size_t tune_grp_b = 0;   // per-warp scratch of the batched kernel (largest candidate)
    int tune_warps = 0;      // resident warps of the batched kernel (largest candidate)
    struct Done {
        pacc_result r;
        std::vector<int32_t> max_z;
        std::vector<double> post_z;
        std::vector<double> tr_d;
        std::vector<int8_t> tr_z;
        std::vector<int8_t> end_z;
    };
    std::vector<Done> done;
    size_t done_head = 0;
    pacc_counters counters;
    // persistent device buffers (grown on demand)
    void* d_ws = nullptr; size_t ws_cap = 0;
    void* d_blob = nullptr; size_t blob_cap = 0;
    void* d_misc = nullptr; size_t misc_cap = 0;
    Server srv;
    StreamServer ss;
    GbgcServer gs;
};

static std::string g_create_error;

static bool cuda_ok(pacc_ctx* c, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    if (c) c->err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

static bool grow(pacc_ctx* c, void** p, size_t* cap, size_t need) {
    if (*cap >= need) return true;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    size_t n = std::max(need, (size_t)(*cap * 3 / 2));
    if (!cuda_ok(c, cudaMalloc(p, n), "cudaMalloc")) return false;
    *cap = n;
    return true;
}

// Eval2 and Output_init (bpp_c2.cpp:29-286, 603-660) of one element from its
// device traces: trd [3][4][T], tzb [3][T][2][N] (Z then B), mzb [3][2][N]
// (Max_Z then Max_B), mll [3].  Fills r and the buffers r points to.
static void gbgc_finish(const pacc_gbgc_opts& g, int N, const GbgcElem& E, const double* trd, const int8_t* tzb,
                        const int8_t* mzb, const double* mll, pacc_gbgc_result& r) {
    const int T = g.burnin + g.mcmc;
    for (int m = 0; m < 3; m++) {
        const double* d = trd + (size_t)m * 4 * T;
        const int8_t* zb = tzb + (size_t)m * T * 2 * N;
        const int8_t* mz = mzb + (size_t)m * 2 * N;
        const int8_t* mb = mz + N;
        r.max_loglik[m] = mll[m];
        const double ll = gbgc_eval2(m, T, g.burnin, g.mcmc, N, E.nodes, E.missing, d, zb,
                                     zb + N, 2 * (size_t)N, mz, r.max_loglik[m]);
        if (m == 0) r.loglik_null = ll;
        else if (m == 2) r.loglik_res = ll;
        else r.loglik_all = ll;
        // Output_init (bpp_c2.cpp:603-660)
        for (int q = 0; q < 3; q++) {
            std::vector<double> v(d + (q + 1) * T, d + (q + 2) * T);
            std::sort(v.begin() + g.burnin, v.end());
            r.rates[m][q] = v[v.size() / 2];
        }
        for (int s = 0; s < N; s++) {
            int cz[4] = {0, 0, 0, 0}, cb = 0;
            for (int it = g.burnin; it < T; it++) {
                cz[zb[(size_t)it * 2 * N + s] + 1]++;
                cb += zb[(size_t)it * 2 * N + N + s];
            }
            if (E.missing[s]) cz[0] = g.mcmc;
            if (r.post_b) r.post_b[(size_t)m * N + s] = (double)cb / g.mcmc;
            if (r.post_z)
                for (int q = 0; q < 4; q++) r.post_z[((size_t)m * N + s) * 4 + q] = (double)cz[q] / g.mcmc;
            if (r.max_z) r.max_z[(size_t)m * N + s] = mz[s];
            if (r.max_b) r.max_b[(size_t)m * N + s] = mb[s];
        }
        if (r.trace) {
            const int Wd = 4 + 2 * N;
            for (int it = 0; it < T; it++) {
                double* row = r.trace + ((size_t)m * T + it) * Wd;
                for (int q = 0; q < 4; q++) row[q] = d[(size_t)q * T + it];
                for (int s = 0; s < N; s++) {
                    row[4 + s] = zb[(size_t)it * 2 * N + N + s];
                    row[4 + N + s] = zb[(size_t)it * 2 * N + s];
                }
            }
        }
    }
}


// ---- gBGC serving (pacc_gbgc_submit / pacc_gbgc_poll / pacc_gbgc_sync) ----

static double gbgc_now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static size_t gbgc_blob_cap(int S, int N, int GGp) {
    return (size_t)72 * N + (size_t)16 * S + (size_t)S * GGp + 1024;
}

static size_t gbgc_out_bytes(int N, int T) {
    return (size_t)3 * 4 * T * 8 + (size_t)3 * T * 2 * N + (size_t)3 * 2 * N + 3 * 8 + 8;
}

static int gbgc_serve_setup(pacc_ctx* c, const pacc_gbgc_opts& g, int GGp_need) {
    GbgcServer& v = c->gs;
    const HostModel& M = c->M;
    const int S = M.S, N = M.N;
    v.N = N;
    v.T = g.burnin + g.mcmc;
    v.GGp_cap = std::max(512, (GGp_need + 255) & ~255);
    v.prec = (c->o.precision == PACC_FP32 || c->o.precision == PACC_FP32_WARP) ? 1 : 0;
    v.regs = c->o.register_budget == 168 ? 168 : 96;
    v.smem = gbgc_chain_smem(N, v.prec);
    const int per_sm = gbgc_chain_occupancy(v.prec, v.regs, v.smem);
    if (per_sm <= 0) { c->err = "gbgc serving: the chain kernel does not fit on an SM"; return PACC_ECUDA; }
    v.grid = c->n_sm * per_sm;
    v.g = g;
    v.target.assign(g.target, g.target + g.n_target);
    v.g.target = v.target.data();
    v.blob_cap = (gbgc_blob_cap(S, N, v.GGp_cap) + 255) & ~(size_t)255;
    v.out_b = (gbgc_out_bytes(N, v.T) + 255) & ~(size_t)255;
    const GbgcWs W = GbgcWs::make(N, S - 1, v.GGp_cap, gbgc_chain_warps(), v.prec ? 4 : 8);
    // slots: two queued elements per resident CTA, within the memory budget
    size_t budget = (size_t)c->o.memory_budget_bytes;
    if (budget == 0) {   // as the plain path: a quarter of the free device memory
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        budget = fr / 4;
    }
    const size_t fixed = W.total * v.grid + 4096;
    const size_t per_slot = sizeof(GbgcElemHdr) + v.blob_cap + v.out_b;
    if (budget <= fixed + per_slot) { c->err = "gbgc serving: memory budget too small"; return PACC_OOM; }
    const size_t want = c->o.max_resident > 0 ? (size_t)c->o.max_resident : (size_t)2 * v.grid;
    v.ns = (int)std::min<size_t>(want, (budget - fixed) / per_slot);
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t o_hdr = 0, o_blob = up(sizeof(GbgcElemHdr) * v.ns), o_out = up(o_blob + v.blob_cap * v.ns);
    // outputs by kind, as the kernel writes them: tr_d [ns][3][4][T], tr_zb [ns][3][T][2][N],
    // max_zb [ns][3][2][N], max_ll [ns][3], status [ns]
    const size_t o_trd = o_out, o_tzb = up(o_trd + (size_t)v.ns * 3 * 4 * v.T * 8);
    const size_t o_mzb = up(o_tzb + (size_t)v.ns * 3 * v.T * 2 * N), o_mll = up(o_mzb + (size_t)v.ns * 3 * 2 * N);
    const size_t o_st = up(o_mll + (size_t)v.ns * 3 * 8), o_out_end = up(o_st + (size_t)v.ns * 4);
    const size_t o_tgt = up(o_out_end), o_head = up(o_tgt + N), o_idle = o_head + 128, o_phase = o_head + 192;
    const size_t o_ws = up(o_head + 256), total = up(o_ws + W.total * v.grid);
    if (!cuda_ok(c, cudaMalloc((void**)&v.dev, total), "cudaMalloc (gbgc serving)")) return PACC_OOM;
    if (!cuda_ok(c, cudaMemset(v.dev, 0, o_ws), "memset")) return PACC_ECUDA;
    std::vector<uint8_t> tgt(N, 0);
    for (int t : v.target)
        if (t >= 0 && t < N) tgt[t] = 1;
    if (!cuda_ok(c, cudaMemcpy(v.dev + o_tgt, tgt.data(), N, cudaMemcpyHostToDevice), "H2D")) return PACC_ECUDA;
    const size_t map_b = sizeof(int) * (64 + 2 * (size_t)v.ns);
    if (!cuda_ok(c, cudaHostAlloc((void**)&v.h_map, map_b, cudaHostAllocMapped), "cudaHostAlloc")) return PACC_OOM;
    std::memset(v.h_map, 0, map_b);
    int* d_map = nullptr;
    if (!cuda_ok(c, cudaHostGetDevicePointer((void**)&d_map, v.h_map, 0), "cudaHostGetDevicePointer")) return PACC_ECUDA;
    v.h_tail = v.h_map;
    v.h_stop = v.h_map + 1;
    v.h_qslot = v.h_map + 64;
    v.h_done = v.h_map + 64 + v.ns;
    v.h_stage_cap = 8 * (v.blob_cap + sizeof(GbgcElemHdr));
    v.out_chunk = (int)std::max<size_t>(1, std::min<size_t>(v.ns, ((size_t)256 << 20) / v.out_b));
    if (!cuda_ok(c, cudaMallocHost((void**)&v.h_stage, v.h_stage_cap), "cudaMallocHost") ||
        !cuda_ok(c, cudaMallocHost((void**)&v.h_out, v.out_b * v.out_chunk), "cudaMallocHost"))
        return PACC_OOM;
    if (!cuda_ok(c, cudaStreamCreateWithFlags(&v.copy, cudaStreamNonBlocking), "stream") ||
        !cuda_ok(c, cudaEventCreate(&v.ev_done), "event") ||
        !cuda_ok(c, cudaEventCreate(&v.ev0), "event"))
        return PACC_ECUDA;
    v.d_hdr = (GbgcElemHdr*)(v.dev + o_hdr);
    v.d_blob = v.dev + o_blob;
    v.d_out = v.dev + o_out;
    v.d_idle = (unsigned long long*)(v.dev + o_idle);
    GbgcChainParams& p = v.p;
    std::memset(&p, 0, sizeof(p));
    p.hdr = v.d_hdr;
    p.blob = (const uint8_t*)v.d_blob;
    p.n_elem = v.ns;
    p.T = v.T; p.burn = g.burnin; p.mcmc = g.mcmc; p.seed = g.seed; p.chain = g.chain;
    p.conserve_rate = g.conserve_rate; p.acce_rate = g.acce_rate; p.init_gc = g.init_gc;
    p.ca = g.conserve_prior_a; p.cb = g.conserve_prior_b;
    p.na = g.acce_prior_a; p.nb = g.acce_prior_b; p.nshift = g.acce_prior_shift;
    p.gca = g.gc_prior_a; p.gcb = g.gc_prior_b; p.gcc = g.gc_prior_c;
    p.lrate = g.prep_lrate; p.grate = g.prep_grate; p.c2m = g.cons_to_mis; p.nc2m = g.ncons_to_mis;
    p.prop_c = g.prop_c; p.prop_n = g.prop_n; p.prop_gc = g.prop_gc;
    std::memcpy(p.Q0, M.rate, sizeof(p.Q0));
    std::memcpy(p.pi, M.pi, sizeof(p.pi));
    p.target = (const uint8_t*)(v.dev + o_tgt);
    p.ws = v.dev + o_ws;
    p.ws_stride = W.total;
    p.N_max = N; p.n_int_max = S - 1; p.GGp_max = v.GGp_cap;
    p.tr_d = (double*)(v.dev + o_trd);
    p.tr_zb = (int8_t*)(v.dev + o_tzb);
    p.max_zb = (int8_t*)(v.dev + o_mzb);
    p.max_ll = (double*)(v.dev + o_mll);
    p.status = (int32_t*)(v.dev + o_st);
    p.stream = 1;
    p.q_head = (int*)(v.dev + o_head);
    p.q_tail = d_map;
    p.q_stop = d_map + 1;
    p.q_slot = d_map + 64;
    p.q_cap = v.ns;
    p.done_flag = d_map + 64 + v.ns;
    p.idle_ns = c->o.serve_idle_ns > 0 ? c->o.serve_idle_ns : 30000000000ll;
    p.idle_exits = v.d_idle;
    p.phase = (unsigned long long*)(v.dev + o_phase);   // 8 counters in the zeroed head block
    p.flop = (unsigned long long*)(v.dev + o_head + 160);
    v.free_slots.clear();
    for (int i = v.ns - 1; i >= 0; i--) v.free_slots.push_back(i);
    v.busy.assign(v.ns, 0);
    v.slot_no.assign(v.ns, 0);
    v.slot_t0.assign(v.ns, 0);
    v.slot_elem.assign(v.ns, GbgcElem());
    v.tail = 0;
    v.resident = 0;
    v.ready = true;
    return PACC_OK;
}

// Admit queued elements into free slots, publish them, and (re)launch the
// persistent kernel when it is not running.
static int gbgc_pump(pacc_ctx* c) {
    GbgcServer& v = c->gs;
    while (!v.free_slots.empty() && !v.queue.empty()) {
        // one staging round: up to 8 elements
        std::vector<int> adm;
        size_t off = 0;
        while (!v.free_slots.empty() && !v.queue.empty() && adm.size() < 8) {
            GbgcServer::Pending& q = v.queue.front();
            const int slot = v.free_slots.back();
            v.free_slots.pop_back();
            q.H.blob_off = (int64_t)slot * (int64_t)v.blob_cap;
            std::memcpy(v.h_stage + off, &q.H, sizeof(GbgcElemHdr));
            std::memcpy(v.h_stage + off + sizeof(GbgcElemHdr), q.blob.data(), q.blob.size());
            bool ok = cuda_ok(c, cudaMemcpyAsync(v.d_blob + (size_t)slot * v.blob_cap, v.h_stage + off + sizeof(GbgcElemHdr),
                                                 q.blob.size(), cudaMemcpyHostToDevice, v.copy), "H2D (gbgc admission)") &&
                      cuda_ok(c, cudaMemcpyAsync(v.d_hdr + slot, v.h_stage + off, sizeof(GbgcElemHdr),
                                                 cudaMemcpyHostToDevice, v.copy), "H2D (gbgc admission)");
            if (!ok) return PACC_ECUDA;
            off += (sizeof(GbgcElemHdr) + q.blob.size() + 255) & ~(size_t)255;
            v.slot_no[slot] = q.no;
            v.slot_t0[slot] = q.t0;
            q.E.masks.clear();
            q.E.masks.shrink_to_fit();
            v.slot_elem[slot] = std::move(q.E);
            v.busy[slot] = 1;
            adm.push_back(slot);
            v.queue.pop_front();
        }
        if (!cuda_ok(c, cudaStreamSynchronize(v.copy), "gbgc admission")) return PACC_ECUDA;
        for (int slot : adm) {
            v.h_done[slot] = 0;
            v.h_qslot[v.tail % v.ns] = slot;
            v.tail++;
        }
        __sync_synchronize();
        *v.h_tail = v.tail;
        v.resident += (int)adm.size();
    }
    if (v.resident > 0) {
        const bool exited = v.running && cudaEventQuery(v.ev_done) == cudaSuccess;
        if (exited) {   // the blocks left on the idle bound: count the launch's time
            float ms = 0;
            if (cudaEventElapsedTime(&ms, v.ev0, v.ev_done) == cudaSuccess) c->counters.kernel_ms += ms;
            v.running = false;
        }
        if (!v.running) {
            *v.h_stop = 0;
            if (!cuda_ok(c, cudaEventRecord(v.ev0, c->stream), "event") ||
                !cuda_ok(c, launch_gbgc_chain(v.p, v.grid, v.smem, v.prec, v.regs, c->stream), "gbgc serving launch") ||
                !cuda_ok(c, cudaEventRecord(v.ev_done, c->stream), "event"))
                return PACC_ECUDA;
            v.running = true;
            v.launches++;
        }
    }
    return PACC_OK;
}

// Collect finished slots: their outputs to the host, Eval2 and the tables.
static int gbgc_collect(pacc_ctx* c) {
    GbgcServer& v = c->gs;
    std::vector<int> fin;
    for (int s = 0; s < v.ns; s++)
        if (v.busy[s] && v.h_done[s]) fin.push_back(s);
    const int N = v.N, T = v.T;
    for (size_t a = 0; a < fin.size(); a += v.out_chunk) {
        const size_t nb = std::min(fin.size() - a, (size_t)v.out_chunk);
        const size_t b_trd = (size_t)3 * 4 * T * 8, b_tzb = (size_t)3 * T * 2 * N, b_mzb = (size_t)3 * 2 * N;
        for (size_t k = 0; k < nb; k++) {
            const size_t sl = (size_t)fin[a + k];
            char* h = v.h_out + k * v.out_b;
            const bool ok =
                cuda_ok(c, cudaMemcpyAsync(h, (const char*)v.p.tr_d + sl * b_trd, b_trd, cudaMemcpyDeviceToHost, v.copy), "D2H") &&
                cuda_ok(c, cudaMemcpyAsync(h + b_trd, (const char*)v.p.tr_zb + sl * b_tzb, b_tzb, cudaMemcpyDeviceToHost, v.copy), "D2H") &&
                cuda_ok(c, cudaMemcpyAsync(h + b_trd + b_tzb, (const char*)v.p.max_zb + sl * b_mzb, b_mzb, cudaMemcpyDeviceToHost, v.copy), "D2H") &&
                cuda_ok(c, cudaMemcpyAsync(h + b_trd + b_tzb + b_mzb, (const char*)v.p.max_ll + sl * 24, 24, cudaMemcpyDeviceToHost, v.copy), "D2H");
            if (!ok) return PACC_ECUDA;
        }
        if (!cuda_ok(c, cudaStreamSynchronize(v.copy), "gbgc results")) return PACC_ECUDA;
        std::vector<GbgcServer::Done> got(nb);
        const double t_done = gbgc_now();
        auto work = [&](size_t k) {
            const int slot = fin[a + k];
            GbgcServer::Done& d = got[k];
            std::memset(&d.r, 0, sizeof(d.r));
            d.max_z.resize(3 * N);
            d.max_b.resize(3 * N);
            d.post_b.resize(3 * N);
            d.post_z.resize(12 * N);
            d.r.max_z = d.max_z.data();
            d.r.max_b = d.max_b.data();
            d.r.post_b = d.post_b.data();
            d.r.post_z = d.post_z.data();
            const char* o = v.h_out + k * v.out_b;
            const double* trd = (const double*)o;
            const int8_t* tzb = (const int8_t*)(o + (size_t)3 * 4 * T * 8);
            const int8_t* mzb = tzb + (size_t)3 * T * 2 * N;
            double mll[3];
            std::memcpy(mll, mzb + (size_t)3 * 2 * N, sizeof(mll));
            d.r.element_no = v.slot_no[slot];
            d.r.status = PACC_OK;
            d.r.root = v.slot_elem[slot].root;
            gbgc_finish(v.g, N, v.slot_elem[slot], trd, tzb, mzb, mll, d.r);
            d.r.device_ms = (t_done - v.slot_t0[slot]) * 1e3;   // submit to collection
            d.r.max_z = nullptr; d.r.max_b = nullptr; d.r.post_b = nullptr; d.r.post_z = nullptr;
        };
        const int nth = std::max(1, std::min((int)nb, std::min(16, (int)std::thread::hardware_concurrency())));
        std::atomic<size_t> next(0);
        std::vector<std::thread> th;
        for (int t = 0; t < nth; t++)
            th.emplace_back([&]() { for (size_t k = next++; k < nb; k = next++) work(k); });
        for (auto& t : th) t.join();
        for (size_t k = 0; k < nb; k++) {
            const int slot = fin[a + k];
            v.done.push_back(std::move(got[k]));
            v.busy[slot] = 0;
            v.h_done[slot] = 0;
            v.free_slots.push_back(slot);
            v.resident--;
        }
    }
    return PACC_OK;
}


static void gbgc_serve_teardown(pacc_ctx* c) {
    GbgcServer& v = c->gs;
    if (!v.ready) return;
    if (v.h_stop) *v.h_stop = 1;
    cudaStreamSynchronize(c->stream);
    if (v.dev) cudaFree(v.dev);
    if (v.h_map) cudaFreeHost(v.h_map);
    if (v.h_stage) cudaFreeHost(v.h_stage);
    if (v.h_out) cudaFreeHost(v.h_out);
    if (v.copy) cudaStreamDestroy(v.copy);
    if (v.ev_done) cudaEventDestroy(v.ev_done);
    if (v.ev0) cudaEventDestroy(v.ev0);
    std::deque<GbgcServer::Done> keep = std::move(v.done);
    const long long launches = v.launches;
    v = GbgcServer();
    v.done = std::move(keep);
    v.launches = launches;
}

static bool gbgc_same_opts(const pacc_gbgc_opts& a, const GbgcServer& v) {
    pacc_gbgc_opts x = a, y = v.g;
    x.target = nullptr; y.target = nullptr;
    if (std::memcmp(&x, &y, sizeof(x)) != 0) return false;
    if (a.n_target != (int)v.target.size()) return false;
    for (int i = 0; i < a.n_target; i++)
        if (a.target[i] != v.target[i]) return false;
    return true;
}

extern "C" {

void pacc_default_opts(pacc_opts* o) {
    std::memset(o, 0, sizeof(*o));
    o->burnin = 200; o->mcmc = 800; o->adapt_freq = 500; o->seed = 5;
    o->init_conserve_rate = 0.5; o->init_acce_rate = 1.0;
    o->conserve_prior_a = 5; o->conserve_prior_b = 0.04;
    o->acce_prior_a = 10; o->acce_prior_b = 0.2;
    o->ropt = 1; o->cub = 1; o->nlb = 0.6;
    o->init_lrate = 0.3; o->init_lrate2 = 0.1; o->init_grate = 0.5;
    o->hyper_lrate_a = 1; o->hyper_lrate_b = 9;
    o->hyper_grate_a = 3; o->hyper_grate_b = 1;
    o->hyper_lrate2_a = 1; o->hyper_lrate2_b = 9;
    o->conserve_prop = 0.8; o->gap_prop = 0.8; o->cons_to_mis = 0.01;
    o->gapchar = '-'; o->prune_tree = 0; o->trim_gap_percent = 1; o->min_len = 50; o->indel = 0;
    o->precision = PACC_FP64; o->device = 0; o->memory_budget_bytes = 0; o->max_resident = 0;
    o->sweeps_per_launch = 0; o->trace_iters = 0; o->block_threads = 0; o->use_graphs = 1;
    o->columns_per_lane = 0;
    o->chain = 0;
}

// The device model (eigensystem, priors, options) lives in constant memory,
// one copy per device.  A context uploads its own before it launches when
// another context's model is there.  Contexts that share a device are driven
// from one host thread at a time (every entry point returns with its work done).
static std::mutex g_model_mu;
static const pacc_ctx* g_model_owner[64];

static bool ensure_model(pacc_ctx* c) {
    std::lock_guard<std::mutex> lk(g_model_mu);
    const int d = c->device;
    if (d >= 0 && d < 64 && g_model_owner[d] == c) return true;
    // a kernel of the context whose model is there may still run (serving):
    // its idle blocks are asked to return, then its launch is waited for
    if (d >= 0 && d < 64 && g_model_owner[d] && g_model_owner[d]->stream) {
        if (g_model_owner[d]->ss.h_stop) *g_model_owner[d]->ss.h_stop = 1;
        cudaStreamSynchronize(g_model_owner[d]->stream);
    }
    if (!cuda_ok(c, set_model(c->M.dm, c->stream), "set_model") ||
        !cuda_ok(c, set_model_batch(c->M.dm, c->stream), "set_model_batch") ||
        !cuda_ok(c, cudaStreamSynchronize(c->stream), "set_model"))
        return false;
    if (d >= 0 && d < 64) g_model_owner[d] = c;
    return true;
}

pacc_ctx* pacc_create(const pacc_model* model, const pacc_opts* opts, int* status) {
    auto fail = [&](int st, const std::string& msg) -> pacc_ctx* {
        g_create_error = msg;
        if (status) *status = st;
        return nullptr;
    };
    if (!model || !opts) return fail(PACC_EINVAL, "null model or opts");
    const int S = model->n_species;
    if (S < 2 || S > 256) return fail(PACC_EINVAL, "n_species must be in [2, 256]");
    if (opts->indel != 0) return fail(PACC_EUNSUPPORTED, "INDEL > 0 (five-state model) is not supported");
    if (opts->chain < 0) return fail(PACC_EINVAL, "chain must be >= 0");
    if (opts->chain > 0 && opts->precision != PACC_FP64 && opts->precision != PACC_FP32)
        return fail(PACC_EUNSUPPORTED, "a later chain (chain > 0) needs PACC_FP64 or PACC_FP32");
    if (opts->sample_hyper &&
        ((opts->precision != PACC_FP64 && opts->precision != PACC_FP32) || opts->sweeps_per_launch > 0))
        return fail(PACC_EUNSUPPORTED, "SAMPLE_HYPER chains need PACC_FP64 or PACC_FP32 without serving");
    if (opts->mcmc < 1 || opts->burnin < 0 || opts->adapt_freq < 1)
        return fail(PACC_EINVAL, "MCMC must be >= 1, BURNIN >= 0, ADAPT_FREQ >= 1");
    if (opts->register_budget != 0 && opts->register_budget != 128 && opts->register_budget != 168 &&
        opts->register_budget != 255)
        return fail(PACC_EINVAL, "register_budget must be 0, 128, 168 or 255");
    if (opts->block_threads < 0 || opts->block_threads > 256 || opts->block_threads % 32 != 0)
        return fail(PACC_EINVAL, "block_threads must be 0 or a multiple of 32 up to 256");
    if (opts->serve_idle_ns < 0) return fail(PACC_EINVAL, "serve_idle_ns must be >= 0");
    pacc_ctx* c = new pacc_ctx();
    c->o = *opts;
    HostModel& M = c->M;
    M.S = S;
    M.N = 2 * S - 1;
    const int N = M.N;
    M.ch0.assign(N, -1); M.ch1.assign(N, -1); M.parent.assign(N, -1);
    M.dist.assign(model->distances, model->distances + N);
    for (int i = 0; i < N; i++) {
        int a = model->children[2 * i], b = model->children[2 * i + 1];
        if ((i < S) != (a < 0) || (a < 0) != (b < 0) || a >= N || b >= N) {
            delete c;
            return fail(PACC_EINVAL, "children[] is not a binary tree with leaves 0..S-1");
        }
        M.ch0[i] = a; M.ch1[i] = b;
        if (a >= 0) M.parent[a] = i;
        if (b >= 0) M.parent[b] = i;
    }
    for (int i = 0; i < N - 1; i++)
        if (M.parent[i] < 0) { delete c; return fail(PACC_EINVAL, "node without parent"); }
    {
        // pending partials of a stack-order prune of the full tree (the
        // child needing more first, Sethi-Ullman): an element's pruned tree
        // is a minor of the full tree and never needs more
        std::vector<int> need(N, 0);
        for (int s = S; s < N; s++) {
            const int a = M.ch0[s], b = M.ch1[s];
            const int na = a >= S ? need[a] : 0, nb = b >= S ? need[b] : 0;
            if (a < S && b < S) need[s] = 1;
            else if (a < S) need[s] = std::max(nb, 1);
            else if (b < S) need[s] = std::max(na, 1);
            else need[s] = std::max(std::max(na, nb), 1 + std::min(na, nb));
        }
        c->stack_cap = std::max(1, need[N - 1]);
    }
    M.outgroup.assign(model->outgroup, model->outgroup + model->n_outgroup);
    M.conserve.assign(model->conserve, model->conserve + model->n_conserve);
    // upper / upper_conserve (getUppertree, bpp.cpp:486-504)
    M.upper.assign(N, 0);
    M.upper_conserve.assign(N, 0);
    auto mark = [&](const std::vector<int>& grp, std::vector<char>& out) {
        for (int p : grp) {
            if (p < 0 || p >= N) continue;
            while (p != N - 1 && p >= 0) { out[p] = 1; p = M.parent[p]; }
        }
        out[N - 1] = 1;
    };
    mark(M.outgroup, M.upper);
    mark(M.conserve, M.upper_conserve);
    // eigensystem (bpp.hpp:357-362)
    double lam[4], V[16], Vi[16];
    int est = pacc_eigen::decompose(4, model->rate_matrix, lam, V, Vi);
    if (est != pacc_eigen::EIG_OK) {
        delete c;
        return fail(PACC_EINVAL, est == pacc_eigen::EIG_COMPLEX ? "RATE_MAT has complex eigenvalues"
                                                                : "RATE_MAT eigendecomposition failed");
    }
    DevModel& dm = M.dm;
    std::memset(&dm, 0, sizeof(dm));
    dm.S = S; dm.N = N;
    std::memcpy(M.rate, model->rate_matrix, sizeof(M.rate));
    for (int i = 0; i < 4; i++) {
        dm.lam[i] = lam[i];
        dm.pi[i] = model->pi[i];
        M.pi[i] = model->pi[i];
        dm.log_pi[i] = std::log(model->pi[i]);
        for (int j = 0; j < 4; j++) {
            dm.evec[i * 4 + j] = V[j * 4 + i];
            dm.einv[i * 4 + j] = Vi[j * 4 + i];
        }
    }
    dm.burnin = opts->burnin; dm.mcmc = opts->mcmc; dm.adapt_freq = opts->adapt_freq; dm.ropt = opts->ropt;
    dm.seed = opts->seed;
    dm.init_c = opts->init_conserve_rate; dm.init_n = opts->init_acce_rate;
    dm.cprior_a = opts->conserve_prior_a; dm.cprior_b = opts->conserve_prior_b;
    dm.nprior_a = opts->acce_prior_a; dm.nprior_b = opts->acce_prior_b;
    dm.cub = opts->cub; dm.nlb = opts->nlb;
    dm.init_l = opts->init_lrate; dm.init_l2 = opts->init_lrate2; dm.init_g = opts->init_grate;
    dm.la = opts->hyper_lrate_a; dm.lb = opts->hyper_lrate_b;
    dm.ga = opts->hyper_grate_a; dm.gb = opts->hyper_grate_b;
    dm.l2a = opts->hyper_lrate2_a; dm.l2b = opts->hyper_lrate2_b;
    dm.cons_to_mis = opts->cons_to_mis;
    dm.trace_iters = opts->trace_iters;
    for (int a = 0; a < 4; a++)
        for (int b = 0; b < 4; b++)
            for (int i = 0; i < 4; i++) dm.a32[(a * 4 + b) * 4 + i] = (float)(dm.einv[a * 4 + i] * dm.evec[i * 4 + b]);
    dm.kc = std::lgamma(dm.cprior_a) + dm.cprior_a * std::log(dm.cprior_b);
    dm.kn = std::lgamma(dm.nprior_a) + dm.nprior_a * std::log(dm.nprior_b);
    c->device = opts->device;
    // Without a usable GPU the context still serves the host-only entry points
    // (pacc_debug_encode); every device call then fails with PACC_ECUDA.
    c->gpu_ok = cuda_ok(c, cudaSetDevice(c->device), "cudaSetDevice") &&
                cuda_ok(c, cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, c->device), "attr") &&
                cuda_ok(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream") &&
                cuda_ok(c, cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking), "stream") &&
                ensure_model(c);
    std::memset(&c->counters, 0, sizeof(c->counters));
    if (status) *status = PACC_OK;
    return c;
}

const char* pacc_last_error(pacc_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

void pacc_destroy(pacc_ctx* c) {
    if (!c) return;
    if (c->gpu_ok && c->stream) {
        cudaSetDevice(c->device);
        if (c->ss.h_stop) *c->ss.h_stop = 1;   // idle serving blocks return
        if (c->gs.h_stop) *c->gs.h_stop = 1;
        cudaStreamSynchronize(c->stream);      // a serving launch may still be in flight
    }
    {
        std::lock_guard<std::mutex> lk(g_model_mu);
        if (c->device >= 0 && c->device < 64 && g_model_owner[c->device] == c) g_model_owner[c->device] = nullptr;
    }
    cudaSetDevice(c->device);
    if (c->d_ws) cudaFree(c->d_ws);
    if (c->d_blob) cudaFree(c->d_blob);
    if (c->d_misc) cudaFree(c->d_misc);
    if (c->srv.gexec) cudaGraphExecDestroy(c->srv.gexec);
    if (c->srv.graph) cudaGraphDestroy(c->srv.graph);
    if (c->srv.dev) cudaFree(c->srv.dev);
    if (c->srv.h_done) cudaFreeHost(c->srv.h_done);
    if (c->srv.h_stage) cudaFreeHost(c->srv.h_stage);
    if (c->srv.ev0) cudaEventDestroy(c->srv.ev0);
    if (c->srv.ev1) cudaEventDestroy(c->srv.ev1);
    if (c->gs.dev) cudaFree(c->gs.dev);
    if (c->gs.h_map) cudaFreeHost(c->gs.h_map);
    if (c->gs.h_stage) cudaFreeHost(c->gs.h_stage);
    if (c->gs.h_out) cudaFreeHost(c->gs.h_out);
    if (c->gs.copy) cudaStreamDestroy(c->gs.copy);
    if (c->gs.ev_done) cudaEventDestroy(c->gs.ev_done);
    if (c->gs.ev0) cudaEventDestroy(c->gs.ev0);
    if (c->ss.dev) cudaFree(c->ss.dev);
    if (c->ss.h_map) cudaFreeHost(c->ss.h_map);
    if (c->ss.h_stage) cudaFreeHost(c->ss.h_stage);
    if (c->ss.h_out) cudaFreeHost(c->ss.h_out);
    if (c->ss.copy) cudaStreamDestroy(c->ss.copy);
    if (c->ss.ev0) cudaEventDestroy(c->ss.ev0);
    if (c->ss.ev1) cudaEventDestroy(c->ss.ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->aux) cudaStreamDestroy(c->aux);
    delete c;
}

// ---------------------------------------------------------------------------
// serving: resident chain slots, continuous admission (batched kernel only)
// ---------------------------------------------------------------------------
// Warp-per-chain layout (pacc_batch.cu) or CTA-per-chain layout (pacc_chain.cu).
static bool batched_layout(const pacc_ctx* c) {
    return c->o.precision == PACC_FP32_WARP || c->o.precision == PACC_FP64_BATCHED;
}
// Serving (continuous batching): sweep-step slots for the warp layout, the
// persistent queue kernel for the CTA layout.
static bool serving(const pacc_ctx* c) { return c->o.sweeps_per_launch > 0; }

static double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------------------
// batched-kernel geometry and the column-count tuner
// ---------------------------------------------------------------------------
struct BatchGeom {
    int C = 1, warps = 4, grid = 1, per_sm = 1;
    size_t wsm = 0, smem = 0, grp_b = 0;
};

// Column counts to consider: the caller's (if compiled), else every compiled one.
static std::vector<int> batch_candidates(const pacc_ctx* c, int prec) {
    int want = c->o.columns_per_lane;
    if (want > 0) {
        while (want > 1 && !batch_supports(prec, want)) want >>= 1;
        return {want};
    }
    std::vector<int> v;
    for (int C = 1; C <= 4; C <<= 1)
        if (batch_supports(prec, C)) v.push_back(C);
    return v;
}

// Warps per CTA (4, 2 or 1) that keep the most warps resident per SM for
// column count C, from the kernel's occupancy (registers and shared memory).
static bool batch_geom(pacc_ctx* c, int prec, int C, int n_int_max, int D, int n_slots, int GGuP, BatchGeom& g) {
    const int N = c->M.N, S = c->M.S;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    g.C = C;
    g.wsm = batch_warp_smem(N, n_int_max, S, D, prec, C);
    int max_smem = 0;
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
    const int wmax = c->o.block_threads > 0 ? std::min(4, std::max(1, c->o.block_threads / 32)) : 4;
    int best = 0;
    for (int w = wmax; w >= 1; w >>= 1) {
        const size_t sm = g.wsm * w;
        if (sm > (size_t)max_smem) continue;
        const int nb = batch_occupancy(prec, C, w, sm);
        if (nb * w > best) { best = nb * w; g.warps = w; g.smem = sm; g.per_sm = nb; }
    }
    if (best == 0) return false;
    g.grid = std::max(1, std::min(c->n_sm * g.per_sm, (std::max(n_slots, 1) + g.warps - 1) / g.warps));
    g.grp_b = al(batch_grp_bytes(c->o.mcmc, n_int_max, prec, GGuP, c->M.N));
    return true;
}

// Tuned column counts, per (device, taxa, precision, stack depth).
static std::mutex g_tune_mu;
static std::map<std::array<int, 4>, int> g_tuned;

static int tuned_columns(const pacc_ctx* c, int prec, int D) {
    auto cands = batch_candidates(c, prec);
    if (cands.size() == 1) return cands[0];
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find({c->device, c->M.S, prec, D});
    return it == g_tuned.end() ? 0 : it->second;
}

// Picks the column count for this batch.  Without a tuned value and with at
// least a device-full of chains, each candidate runs the same sample of
// chains (every k-th element of the batch) for a few sweeps from a fresh
// start and the fastest is kept for every later batch of this shape.  The
// trial launches use the batch's own buffers before they are initialised for
// the real run.
static int tune_columns(pacc_ctx* c, int prec, int D, int n_int_max, int GGuP, const std::vector<int32_t>& elem,
                        BatchParams& p, char* d_elem, char* d_ctr, int& C) {
    C = tuned_columns(c, prec, D);
    if (C > 0) return PACC_OK;
    C = 1;
    const int n_real = elem.empty() || elem[0] < 0 ? 0 : (int)elem.size();
    BatchGeom g1;
    if (!batch_geom(c, prec, 1, n_int_max, D, n_real, GGuP, g1)) return PACC_OK;
    const int n_trial = c->n_sm * g1.per_sm * g1.warps;
    if (n_real < n_trial) return PACC_OK;   // too few chains to fill the device: keep 1, decide later
    std::vector<int32_t> trial(n_trial);
    for (int i = 0; i < n_trial; i++) trial[i] = elem[(size_t)i * n_real / n_trial];
    cudaStream_t st = c->stream;
    if (!cuda_ok(c, cudaMemcpyAsync(d_elem, trial.data(), sizeof(int32_t) * n_trial, cudaMemcpyHostToDevice, st),
                 "H2D trial"))
        return PACC_ECUDA;
    const int save_sweeps = p.sweeps;
    const int save_slots = p.n_slots;
    p.n_slots = n_trial;
    p.sweeps = 6;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 0;
    auto cands = batch_candidates(c, prec);
    for (int rep = 0; rep < 2; rep++) {   // the first round warms the device up
        for (int Cc : cands) {
            BatchGeom g;
            if (!batch_geom(c, prec, Cc, n_int_max, D, n_trial, GGuP, g)) continue;
            float ms = 0;
            bool ok = cuda_ok(c, launch_init_slots(p.slots, (const int32_t*)d_elem, n_trial, st), "trial slots") &&
                      cuda_ok(c, cudaMemsetAsync(d_ctr, 0, 256, st), "trial queue") &&
                      cuda_ok(c, cudaEventRecord(e0, st), "event") &&
                      cuda_ok(c, launch_batch(&p, g.grid, g.warps, g.smem, prec, Cc, st), "trial launch") &&
                      cuda_ok(c, cudaEventRecord(e1, st), "event") &&
                      cuda_ok(c, cudaStreamSynchronize(st), "trial launch") &&
                      cuda_ok(c, cudaEventElapsedTime(&ms, e0, e1), "event");
            if (!ok) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                return PACC_ECUDA;
            }
            if (rep == 1 && (best == 0 || ms < best)) { best = ms; C = Cc; }
        }
        if (cands.size() == 1) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    p.sweeps = save_sweeps;
    p.n_slots = save_slots;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[{c->device, c->M.S, prec, D}] = C;
    return PACC_OK;
}

// Stack depth bound of the unpruned tree: pruning only removes nodes.
static int tree_stack_depth(const HostModel& M) {
    std::vector<int> need(M.N, 0), order, todo{M.N - 1};
    while (!todo.empty()) {  // preorder; reversed below it visits children first
        int s = todo.back();
        todo.pop_back();
        if (s < M.S) continue;
        order.push_back(s);
        todo.push_back(M.ch0[s]);
        todo.push_back(M.ch1[s]);
    }
    for (auto it = order.rbegin(); it != order.rend(); ++it) {
        const int s = *it;
        int a = M.ch0[s], b = M.ch1[s];
        int na = a >= M.S ? need[a] : 0, nb = b >= M.S ? need[b] : 0;
        if (a < M.S && b < M.S) need[s] = 1;
        else if (a < M.S) need[s] = std::max(nb, 1);
        else if (b < M.S) need[s] = std::max(na, 1);
        else need[s] = std::max(std::max(na, nb), 1 + std::min(na, nb));
    }
    return std::max(1, need[M.N - 1]);
}

static int server_setup(pacc_ctx* c, int GG_needed) {
    Server& v = c->srv;
    if (v.ready) return PACC_OK;
    cudaSetDevice(c->device);
    if (!ensure_model(c)) return PACC_ECUDA;
    const int N = c->M.N, S = c->M.S;
    const int T = c->o.burnin + c->o.mcmc;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    v.prec = c->o.precision == PACC_FP32_WARP ? 1 : 0;
    v.D = tree_stack_depth(c->M);
    v.n_int_max = S - 1;
    v.SP = (S + 15) & ~15;
    v.GG_cap = std::max(5120, (GG_needed + 31) & ~31);
    // the column count tuned by an earlier batch of this shape, else 1
    v.C = tuned_columns(c, v.prec, v.D);
    if (v.C <= 0) v.C = 1;
    BatchGeom g;
    if (!batch_geom(c, v.prec, v.C, v.n_int_max, v.D, 1 << 30, v.GG_cap, g)) {
        c->err = "element tree too large for the batched kernel";
        return PACC_EUNSUPPORTED;
    }
    v.warps = g.warps;
    v.smem = g.smem;
    v.grid = g.grid;
    const int n_warps = v.grid * v.warps;
    v.tb = al(topo_bytes(N));
    v.o_prefix = v.tb;
    v.o_codes = al(v.o_prefix + (size_t)(v.GG_cap + 1) * 4);
    v.o_pcodes = al(v.o_codes + (size_t)v.GG_cap * v.SP);
    v.o_pw = al(v.o_pcodes + (size_t)v.GG_cap * v.SP);
    v.o_pof = al(v.o_pw + (size_t)v.GG_cap * 4);
    v.blob_b = al(v.o_pof + (size_t)v.GG_cap * 4);
    v.slot_b = al(batch_slot_bytes(N, T));
    v.grp_b = al(batch_grp_bytes(c->o.mcmc, v.n_int_max, v.prec, v.GG_cap, N));
    v.TI = std::min(c->o.trace_iters, T);
    size_t per_slot = v.blob_b + v.slot_b + sizeof(ElemHeader) + sizeof(SlotState) + sizeof(DevResult) +
                      3 * N * 4 + 3 * N * 4 * 8 + sizeof(double) * 3 * 6 * (size_t)v.TI + (size_t)3 * v.TI * N + 8;
    size_t budget = (size_t)c->o.memory_budget_bytes;
    if (budget == 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        budget = fr / 4;
    }
    // one resident chain per warp: every chain advances in every step, so
    // latency is the chain's own length; more slots would only queue on warps
    int want = c->o.max_resident > 0 ? c->o.max_resident : n_warps;
    size_t fixed = (size_t)n_warps * v.grp_b + (1 << 20);
    if (budget <= fixed + per_slot) { c->err = "memory budget too small for one chain slot"; return PACC_OOM; }
    v.n_slots = (int)std::min<size_t>((size_t)want, (budget - fixed) / per_slot);
    const int ns = v.n_slots;
    size_t o = 0;
    size_t o_hdr = o; o = al(o + sizeof(ElemHeader) * ns);
    size_t o_blob = o; o = al(o + v.blob_b * ns);
    size_t o_slots = o; o = al(o + sizeof(SlotState) * ns);
    size_t o_sws = o; o = al(o + v.slot_b * ns);
    size_t o_grp = o; o = al(o + v.grp_b * n_warps);
    size_t o_res = o; o = al(o + sizeof(DevResult) * ns);
    size_t o_mz = o; o = al(o + sizeof(int32_t) * 3 * N * (size_t)ns);
    size_t o_pz = o; o = al(o + sizeof(double) * 3 * N * 4 * (size_t)ns);
    size_t o_trd = o; o = al(o + sizeof(double) * 3 * 6 * (size_t)v.TI * ns);
    size_t o_trz = o; o = al(o + (size_t)3 * v.TI * N * ns);
    size_t o_cnt = o; o = al(o + sizeof(DevCounters));
    size_t o_ctr = o; o = al(o + 256);
    size_t o_done = o; o = al(o + sizeof(int) * (ns + 1));
    if (!cuda_ok(c, cudaMalloc((void**)&v.dev, o), "cudaMalloc (serving slots)")) return PACC_OOM;
    if (!cuda_ok(c, cudaMallocHost((void**)&v.h_done, sizeof(int) * (ns + 2)), "cudaMallocHost")) return PACC_OOM;
    if (!cuda_ok(c, cudaEventCreate(&v.ev0), "event") || !cuda_ok(c, cudaEventCreate(&v.ev1), "event"))
        return PACC_ECUDA;
    v.d_hdr = (ElemHeader*)(v.dev + o_hdr);
    v.d_blob = v.dev + o_blob;
    v.d_slots = (SlotState*)(v.dev + o_slots);
    v.d_slotws = v.dev + o_sws;
    v.d_grp = v.dev + o_grp;
    v.d_res = (DevResult*)(v.dev + o_res);
    v.d_mz = (int32_t*)(v.dev + o_mz);
    v.d_pz = (double*)(v.dev + o_pz);
    v.d_trd = v.TI > 0 ? (double*)(v.dev + o_trd) : nullptr;
    v.d_trz = v.TI > 0 ? (int8_t*)(v.dev + o_trz) : nullptr;
    v.d_cnt = (DevCounters*)(v.dev + o_cnt);
    v.d_ctr = (int*)(v.dev + o_ctr);
    v.d_done = (int*)(v.dev + o_done);
    cudaStream_t st = c->stream;
    if (!cuda_ok(c, cudaMemsetAsync(v.dev, 0, o, st), "memset slots")) return PACC_ECUDA;
    // every slot starts empty
    std::vector<int32_t> empty(ns, -1);
    int32_t* d_e = nullptr;
    if (!cuda_ok(c, cudaMalloc((void**)&d_e, sizeof(int32_t) * ns), "cudaMalloc") ||
        !cuda_ok(c, cudaMemcpyAsync(d_e, empty.data(), sizeof(int32_t) * ns, cudaMemcpyHostToDevice, st), "H2D") ||
        !cuda_ok(c, launch_init_slots(v.d_slots, d_e, ns, st), "init slots") ||
        !cuda_ok(c, cudaStreamSynchronize(st), "init slots"))
        return PACC_ECUDA;
    cudaFree(d_e);
    std::memset(&v.p, 0, sizeof(v.p));
    v.p.hdr = v.d_hdr;
    v.p.blob = (const uint8_t*)v.d_blob;
    v.p.slots = v.d_slots;
    v.p.n_slots = ns;
    v.p.slot_ws = v.d_slotws;
    v.p.slot_ws_stride = v.slot_b;
    v.p.grp_ws = v.d_grp;
    v.p.grp_ws_stride = v.grp_b;
    v.p.sweeps = c->o.sweeps_per_launch;
    v.p.results = v.d_res;
    v.p.max_z = v.d_mz;
    v.p.post_z = v.d_pz;
    v.p.tr_d = v.d_trd;
    v.p.tr_z = v.d_trz;
    v.p.counters = v.d_cnt;
    v.p.n_done = v.d_ctr;
    v.p.next_slot = v.d_ctr + 32;
    v.p.done_list = v.d_done;
    v.p.n_int_max = v.n_int_max;
    v.p.S_max = S;
    v.p.stack_depth = v.D;
    v.p.GGuP_max = v.GG_cap;
    // the sweep step: reset the queue counters, advance every resident chain,
    // copy the list of chains that finished back to pinned host memory
    auto record = [&](cudaStream_t s2) -> cudaError_t {
        cudaError_t e = cudaMemsetAsync(v.d_ctr, 0, 256, s2);
        if (e == cudaSuccess) e = launch_batch(&v.p, v.grid, v.warps, v.smem, v.prec, v.C, s2);
        if (e == cudaSuccess) e = cudaMemcpyAsync(v.h_done, v.d_ctr, sizeof(int), cudaMemcpyDeviceToHost, s2);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(v.h_done + 1, v.d_done, sizeof(int) * ns, cudaMemcpyDeviceToHost, s2);
        return e;
    };
    // one step over the empty slots outside capture: sets the kernel's
    // shared-memory attribute and checks the launch geometry
    if (!cuda_ok(c, record(st), "first sweep step") || !cuda_ok(c, cudaStreamSynchronize(st), "first sweep step"))
        return PACC_ECUDA;
    if (c->o.use_graphs) {
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) e = record(st);
        cudaError_t e2 = cudaStreamEndCapture(st, &v.graph);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&v.gexec, v.graph, 0);
        if (e != cudaSuccess) {
            cudaGetLastError();
            if (v.graph) { cudaGraphDestroy(v.graph); v.graph = nullptr; }
            v.gexec = nullptr;
        }
    }
    v.free_slots.clear();
    for (int i = ns - 1; i >= 0; i--) v.free_slots.push_back(i);
    v.slot_no.assign(ns, 0);
    v.slot_t0.assign(ns, 0);
    v.resident = 0;
    v.ready = true;
    return PACC_OK;
}

// Move queued elements into free slots.
static int server_admit(pacc_ctx* c) {
    Server& v = c->srv;
    const int N = c->M.N;
    cudaStream_t st = c->stream;
    std::vector<std::pair<int, std::pair<HostElem, double>>> adm;
    while (!v.free_slots.empty() && !v.queue.empty()) {
        int slot = v.free_slots.back();
        v.free_slots.pop_back();
        adm.push_back({slot, std::move(v.queue.front())});
        v.queue.pop_front();
    }
    if (adm.empty()) return PACC_OK;
    // stage every admitted element contiguously in pinned memory, then copy
    auto staged = [&](const HostElem& E) {
        return v.tb + E.prefix.size() * 4 + E.codes_t.size() + E.pcodes_t.size() + E.pw.size() * 4 +
               E.pattern_of.size() * 4 + sizeof(ElemHeader) + sizeof(SlotState) + 64;
    };
    size_t tot = 0;
    for (auto& a : adm) tot += staged(a.second.first);
    if (tot > v.h_stage_cap) {
        if (v.h_stage) cudaFreeHost(v.h_stage);
        v.h_stage = nullptr;
        v.h_stage_cap = 0;
        if (!cuda_ok(c, cudaMallocHost((void**)&v.h_stage, tot * 2), "cudaMallocHost")) return PACC_OOM;
        v.h_stage_cap = tot * 2;
    }
    char* hs = v.h_stage;
    size_t off = 0;
    for (auto& a : adm) {
        const int slot = a.first;
        const HostElem& E = a.second.first;
        char* reg = v.d_blob + (size_t)slot * v.blob_b;
        ElemHeader H;
        std::memset(&H, 0, sizeof(H));
        H.GG = E.GG; H.GGp = E.GGp; H.root = E.root; H.n_nodes = E.n_nodes; H.n_int = E.n_int;
        H.n_hlev = E.n_hlev; H.n_dlev = E.n_dlev; H.tg_draws = E.tg_draws; H.stack_depth = E.stack_depth;
        H.element_no = E.no;
        H.SP = v.SP;
        H.topo_off = (int64_t)(reg - v.d_blob);
        H.prefix_off = H.topo_off + (int64_t)v.o_prefix;
        H.codes_t_off = H.topo_off + (int64_t)v.o_codes;
        H.codes_off = H.codes_t_off;
        H.tg_off = 0;
        H.GGu = E.GGu;
        H.pcodes_off = H.topo_off + (int64_t)v.o_pcodes;
        H.pw_off = H.topo_off + (int64_t)v.o_pw;
        H.pof_off = H.topo_off + (int64_t)v.o_pof;
        char* p0 = hs + off;
        std::memcpy(p0, E.topo.data(), E.topo.size() * 2);
        std::memcpy(p0 + ((E.topo.size() * 2 + 15) & ~(size_t)15), E.dist2.data(), N * 8);
        char* p1 = p0 + v.tb;
        std::memcpy(p1, E.prefix.data(), E.prefix.size() * 4);
        char* p2 = p1 + E.prefix.size() * 4;
        std::memcpy(p2, E.codes_t.data(), E.codes_t.size());
        char* p5 = p2 + E.codes_t.size();
        std::memcpy(p5, E.pcodes_t.data(), E.pcodes_t.size());
        char* p6 = p5 + E.pcodes_t.size();
        std::memcpy(p6, E.pw.data(), E.pw.size() * 4);
        char* p7 = p6 + E.pw.size() * 4;
        std::memcpy(p7, E.pattern_of.data(), E.pattern_of.size() * 4);
        char* p3 = p7 + E.pattern_of.size() * 4;
        std::memcpy(p3, &H, sizeof(H));
        SlotState S0;
        std::memset(&S0, 0, sizeof(S0));
        S0.elem = slot;
        S0.phase = 0;  // PH_INIT
        char* p4 = p3 + sizeof(H);
        std::memcpy(p4, &S0, sizeof(S0));
        bool ok = cuda_ok(c, cudaMemcpyAsync(reg, p0, v.tb, cudaMemcpyHostToDevice, st), "H2D topo") &&
                  cuda_ok(c, cudaMemcpyAsync(reg + v.o_prefix, p1, E.prefix.size() * 4, cudaMemcpyHostToDevice, st), "H2D prefix") &&
                  cuda_ok(c, cudaMemcpyAsync(reg + v.o_codes, p2, E.codes_t.size(), cudaMemcpyHostToDevice, st), "H2D codes") &&
                  cuda_ok(c, cudaMemcpyAsync(reg + v.o_pcodes, p5, E.pcodes_t.size(), cudaMemcpyHostToDevice, st), "H2D patterns") &&
                  cuda_ok(c, cudaMemcpyAsync(reg + v.o_pw, p6, E.pw.size() * 4, cudaMemcpyHostToDevice, st), "H2D weights") &&
                  cuda_ok(c, cudaMemcpyAsync(reg + v.o_pof, p7, E.pattern_of.size() * 4, cudaMemcpyHostToDevice, st), "H2D pattern map") &&
                  cuda_ok(c, cudaMemcpyAsync(v.d_hdr + slot, p3, sizeof(H), cudaMemcpyHostToDevice, st), "H2D header") &&
                  cuda_ok(c, cudaMemcpyAsync(v.d_slots + slot, p4, sizeof(S0), cudaMemcpyHostToDevice, st), "H2D slot") &&
                  cuda_ok(c, cudaMemsetAsync(v.d_res + slot, 0, sizeof(DevResult), st), "memset result");
        if (!ok) return PACC_ECUDA;
        off += staged(E);
        v.slot_no[slot] = E.no;
        v.slot_t0[slot] = a.second.second;
        v.resident++;
    }
    cudaError_t e = cudaStreamSynchronize(st);
    return cuda_ok(c, e, "admission") ? PACC_OK : PACC_ECUDA;
}

// One sweep step over the resident chains; finished chains become results.
// Retires the sweep in flight, if any: waits for it, copies the finished
// chains' results back and frees their slots.
static int server_retire(pacc_ctx* c) {
    Server& v = c->srv;
    if (!v.inflight) return PACC_OK;
    v.inflight = false;
    const int N = c->M.N;
    cudaStream_t st = c->stream;
    if (!cuda_ok(c, cudaStreamSynchronize(st), "sweep step")) return PACC_ECUDA;
    float ms = 0;
    cudaEventElapsedTime(&ms, v.ev0, v.ev1);
    v.kernel_ms += ms;
    v.steps++;
    const int nd = v.h_done[0];
    if (nd <= 0) return PACC_OK;
    int clk_khz = 0;
    cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, c->device);
    std::vector<DevResult> res(nd);
    std::vector<int32_t> mz((size_t)nd * 3 * N);
    std::vector<double> pz((size_t)nd * 3 * N * 4);
    for (int i = 0; i < nd; i++) {
        int slot = v.h_done[1 + i];
        cudaMemcpyAsync(&res[i], v.d_res + slot, sizeof(DevResult), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&mz[(size_t)i * 3 * N], v.d_mz + (size_t)slot * 3 * N, sizeof(int32_t) * 3 * N,
                        cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&pz[(size_t)i * 3 * N * 4], v.d_pz + (size_t)slot * 3 * N * 4, sizeof(double) * 3 * N * 4,
                        cudaMemcpyDeviceToHost, st);
    }
    const size_t trd_n = (size_t)3 * 6 * v.TI, trz_n = (size_t)3 * v.TI * N;
    std::vector<double> trd(trd_n * nd);
    std::vector<int8_t> trz(trz_n * nd);
    if (v.TI > 0)
        for (int i = 0; i < nd; i++) {
            int slot = v.h_done[1 + i];
            cudaMemcpyAsync(&trd[trd_n * i], v.d_trd + trd_n * slot, sizeof(double) * trd_n, cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(&trz[trz_n * i], v.d_trz + trz_n * slot, trz_n, cudaMemcpyDeviceToHost, st);
        }
    if (!cuda_ok(c, cudaStreamSynchronize(st), "D2H results")) return PACC_ECUDA;
    const double t = now_ms();
    for (int i = 0; i < nd; i++) {
        int slot = v.h_done[1 + i];
        pacc_ctx::Done d;
        std::memset(&d.r, 0, sizeof(d.r));
        d.r.element_no = v.slot_no[slot];
        d.r.n_nodes = N;
        const DevResult& R = res[i];
        d.r.status = R.status == 0 ? PACC_OK : (R.status == 2 ? PACC_NAN_LIKELIHOOD : PACC_SAMPLER_ERROR);
        for (int m = 0; m < 3; m++) {
            pacc_model_result& mr = d.r.model[m];
            mr.loglik = R.model[m].loglik;
            mr.max_loglik = R.model[m].max_loglik;
            mr.n_rate = R.model[m].rates[0];
            mr.c_rate = R.model[m].rates[1];
            mr.g_rate = R.model[m].rates[2];
            mr.l_rate = R.model[m].rates[3];
            mr.l2_rate = R.model[m].rates[4];
            mr.failure = R.model[m].failure;
            mr.n_configs = R.model[m].n_configs;
        }
        d.r.device_ms = clk_khz > 0 ? R.device_ms / (double)clk_khz : 0.0;
        d.r.latency_ms = t - v.slot_t0[slot];
        d.max_z.assign(mz.begin() + (size_t)i * 3 * N, mz.begin() + (size_t)(i + 1) * 3 * N);
        d.post_z.assign(pz.begin() + (size_t)i * 3 * N * 4, pz.begin() + (size_t)(i + 1) * 3 * N * 4);
        if (v.TI > 0) {
            d.tr_d.assign(trd.begin() + trd_n * i, trd.begin() + trd_n * (i + 1));
            d.tr_z.assign(trz.begin() + trz_n * i, trz.begin() + trz_n * (i + 1));
        }
        c->done.push_back(std::move(d));
        // the slot's device state is PH_DONE, which the kernel skips until re-admission
        v.free_slots.push_back(slot);
        v.resident--;
    }
    return PACC_OK;
}

// One serving step: retire the previous sweep, admit queued elements into the
// free slots, and launch the next sweep (the graph: queue reset, batched
// kernel, copy of the finished-slot list) without waiting for it, so that the
// caller's work until the next step overlaps the device's.
static int server_step(pacc_ctx* c) {
    Server& v = c->srv;
    cudaSetDevice(c->device);
    int st0 = server_retire(c);
    if (st0 != PACC_OK) return st0;
    if (!ensure_model(c)) return PACC_ECUDA;
    st0 = server_admit(c);
    if (st0 != PACC_OK) return st0;
    if (v.resident == 0) return PACC_OK;
    cudaStream_t st = c->stream;
    cudaEventRecord(v.ev0, st);
    cudaError_t e;
    if (v.gexec) e = cudaGraphLaunch(v.gexec, st);
    else {
        e = cudaMemsetAsync(v.d_ctr, 0, 256, st);
        if (e == cudaSuccess) e = launch_batch(&v.p, v.grid, v.warps, v.smem, v.prec, v.C, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(v.h_done, v.d_ctr, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(v.h_done + 1, v.d_done, sizeof(int) * v.n_slots, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaEventRecord(v.ev1, st);
    if (!cuda_ok(c, e, "sweep launch")) return PACC_ECUDA;
    v.inflight = true;
    return PACC_OK;
}

// ---------------------------------------------------------------------------
// packing of elements into one device blob
// ---------------------------------------------------------------------------
// Element data (codes, codes by column, initial Tg, draw prefix, topology and
// branch lengths, site patterns) at 256-byte aligned offsets of one blob, and
// the matching headers.  Returns the blob size.
static size_t pack_elems(const pacc_ctx* c, const std::vector<const HostElem*>& els, std::vector<ElemHeader>& hdr,
                         std::vector<uint8_t>& blob, int& n_int_max, int& GGp_max, int& GGuP_max) {
    const int N = c->M.N, S = c->M.S;
    const int n = (int)els.size();
    hdr.assign(n, ElemHeader());
    size_t off = 0;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    n_int_max = 1; GGp_max = 32; GGuP_max = 32;
    const size_t tb = topo_bytes(N);
    for (int e = 0; e < n; e++) {
        const HostElem& E = *els[e];
        ElemHeader& H = hdr[e];
        std::memset(&H, 0, sizeof(H));
        H.element_no = E.no;
        H.filtered = E.filtered;
        if (E.filtered) continue;
        H.GG = E.GG; H.GGp = E.GGp; H.root = E.root; H.n_nodes = E.n_nodes; H.n_int = E.n_int;
        H.n_hlev = E.n_hlev; H.n_dlev = E.n_dlev; H.tg_draws = E.tg_draws;
        H.stack_depth = E.stack_depth;
        H.codes_off = off; off = al(off + E.codes.size());
        H.codes_t_off = off; off = al(off + E.codes_t.size());
        H.SP = (S + 15) & ~15;
        H.tg_off = off; off = al(off + E.tg0.size());
        H.prefix_off = off; off = al(off + E.prefix.size() * 4);
        H.topo_off = off; off = al(off + tb);
        H.GGu = E.GGu;
        H.pcodes_off = off; off = al(off + E.pcodes_t.size());
        H.pw_off = off; off = al(off + E.pw.size() * 4);
        H.pof_off = off; off = al(off + E.pattern_of.size() * 4);
        n_int_max = std::max(n_int_max, E.n_int);
        GGuP_max = std::max(GGuP_max, (E.GGu + 31) & ~31);
        GGp_max = std::max(GGp_max, E.GGp);
    }
    blob.assign(std::max<size_t>(off, 256), 0);
    for (int e = 0; e < n; e++) {
        const HostElem& E = *els[e];
        if (E.filtered) continue;
        ElemHeader& H = hdr[e];
        std::memcpy(&blob[H.codes_off], E.codes.data(), E.codes.size());
        std::memcpy(&blob[H.codes_t_off], E.codes_t.data(), E.codes_t.size());
        std::memcpy(&blob[H.tg_off], E.tg0.data(), E.tg0.size());
        std::memcpy(&blob[H.prefix_off], E.prefix.data(), E.prefix.size() * 4);
        std::memcpy(&blob[H.topo_off], E.topo.data(), E.topo.size() * 2);
        std::memcpy(&blob[H.topo_off + ((E.topo.size() * 2 + 15) & ~(size_t)15)], E.dist2.data(), N * 8);
        std::memcpy(&blob[H.pcodes_off], E.pcodes_t.data(), E.pcodes_t.size());
        std::memcpy(&blob[H.pw_off], E.pw.data(), E.pw.size() * 4);
        std::memcpy(&blob[H.pof_off], E.pattern_of.data(), E.pattern_of.size() * 4);
    }
    return off;
}

// ---------------------------------------------------------------------------
// launch shape of the CTA-per-chain kernel and its trial-launch tuner
// ---------------------------------------------------------------------------
// A shape is a kernel instance (registers a thread) and a block size; with
// the shared memory of that block size they fix the resident chains per SM.
// Results do not depend on the shape (every column is computed by one thread
// in the same arithmetic, and the column sums are exact), so the tuner may
// pick any of them.
struct ChainShape {
    int variant = 0, BT = 128, per_sm = 0;
};
static const int kChainRegs[3] = {128, 168, 255};
static std::mutex g_shape_mu;
static std::map<std::array<int, 3>, std::array<int, 2>> g_shape_cache;   // (device, S, prec) -> (variant, BT)

static int chain_regs(int prec, int variant) { return prec == 0 ? 255 : kChainRegs[variant]; }

static std::vector<ChainShape> shape_candidates(const pacc_ctx* c, int prec) {
    std::vector<ChainShape> v;
    const int N = c->M.N;
    for (int var = 0; var < chain_variants(prec); var++) {
        if (prec == 1 && c->o.register_budget > 0 && kChainRegs[var] != c->o.register_budget) continue;
        std::vector<int> bts;
        // FP64 partials: 128 threads (two chains per SM); on whole chains of
        // the 43-taxon workload 256 threads (one chain per SM) ran at 0.77x
        // and 64 threads fit no more chains per SM (shared memory)
        if (c->o.block_threads > 0) bts.push_back(c->o.block_threads);
        else if (prec == 0) bts = {128};
        else if (var == 0) bts = {64, 128};
        else if (var == 1) bts = {128};
        else bts = {128, 256};
        for (int bt : bts) {
            if (bt > chain_variant_max_threads(prec, var)) continue;
            ChainShape s;
            s.variant = var;
            s.BT = bt;
            s.per_sm = chain_occupancy(prec, var, bt, smem_bytes(N, bt, prec, c->stack_cap));
            if (s.per_sm > 0) v.push_back(s);
        }
    }
    return v;
}

// Chooses the launch shape once per context: the options' shape if they fix
// it, else the one an earlier context chose for this device, taxon count and
// precision, else the fastest candidate on a short trial (BURNIN 40 + MCMC 80
// per model) over the elements at hand (at least one per SM; with fewer the
// default of 128 threads and the smallest register budget is kept).  A
// shape's speed is its resident chains per SM over the mean device time of
// an element's chain (the kernel's per-element clock): the rate at which a
// long stream of elements goes through, without the tail of the trial batch
// (whose last chains run alone), which favours shapes with fewer chains.
static int choose_shape(pacc_ctx* c, int prec, const std::vector<const HostElem*>& els) {
    if (c->shape_ready) return PACC_OK;
    std::vector<ChainShape> cand = shape_candidates(c, prec);
    if (cand.empty()) {
        c->err = "no kernel instance fits the block_threads / register_budget options";
        return PACC_EINVAL;
    }
    auto take = [&](const ChainShape& s) {
        c->shape_variant = s.variant;
        c->shape_bt = s.BT;
        c->shape_per_sm = s.per_sm;
        c->shape_ready = true;
        return PACC_OK;
    };
    if (cand.size() == 1) return take(cand[0]);
    const std::array<int, 3> key = {c->device, c->M.S, prec};
    {
        std::lock_guard<std::mutex> lk(g_shape_mu);
        auto it = g_shape_cache.find(key);
        if (it != g_shape_cache.end())
            for (const ChainShape& s : cand)
                if (s.variant == it->second[0] && s.BT == it->second[1]) return take(s);
    }
    std::vector<const HostElem*> trial;
    int max_per_sm = 1;
    for (const ChainShape& s : cand) max_per_sm = std::max(max_per_sm, s.per_sm);
    const size_t want = (size_t)c->n_sm * max_per_sm;
    for (const HostElem* E : els)
        if (!E->filtered && trial.size() < want) trial.push_back(E);
    if ((int)trial.size() < c->n_sm) {
        for (const ChainShape& s : cand)
            if (s.variant == 0 && s.BT == 128) return take(s);
        return take(cand[0]);
    }
    const int N = c->M.N;
    const int n = (int)trial.size();
    std::vector<ElemHeader> hdr;
    std::vector<uint8_t> blob;
    int n_int_max, GGp_max, GGuP_max;
    pack_elems(c, trial, hdr, blob, n_int_max, GGp_max, GGuP_max);
    const int tb = 40, tm = 80;
    size_t ws1 = (ws_bytes(n_int_max, GGp_max, tb + tm, tm, N, prec) + 4095) & ~(size_t)4095;
    int grid_max = 1;
    for (const ChainShape& s : cand) grid_max = std::max(grid_max, std::min(n, c->n_sm * s.per_sm));
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t o_hdr = 0, o_res = al(sizeof(ElemHeader) * n), o_mz = al(o_res + sizeof(DevResult) * n),
                 o_pz = al(o_mz + sizeof(int32_t) * 3 * N * (size_t)n),
                 o_cnt = al(o_pz + sizeof(double) * 12 * N * (size_t)n), o_next = al(o_cnt + sizeof(DevCounters)),
                 o_order = al(o_next + 256), o_ws = al(o_order + sizeof(int32_t) * n), total = o_ws + ws1 * grid_max;
    std::vector<int32_t> order(n);
    for (int e = 0; e < n; e++) order[e] = e;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return trial[a]->GG > trial[b]->GG; });
    char* dev = nullptr;
    char* dblob = nullptr;
    if (!cuda_ok(c, cudaMalloc((void**)&dev, total), "cudaMalloc (tuner)")) return PACC_OOM;
    if (!cuda_ok(c, cudaMalloc((void**)&dblob, blob.size()), "cudaMalloc (tuner)")) { cudaFree(dev); return PACC_OOM; }
    cudaStream_t st = c->stream;
    bool ok = cuda_ok(c, cudaMemcpyAsync(dblob, blob.data(), blob.size(), cudaMemcpyHostToDevice, st), "H2D (tuner)") &&
              cuda_ok(c, cudaMemcpyAsync(dev + o_hdr, hdr.data(), sizeof(ElemHeader) * n, cudaMemcpyHostToDevice, st),
                      "H2D (tuner)") &&
              cuda_ok(c, cudaMemcpyAsync(dev + o_order, order.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st),
                      "H2D (tuner)");
    ChainParams p;
    std::memset(&p, 0, sizeof(p));
    p.hdr = (const ElemHeader*)(dev + o_hdr);
    p.blob = (const uint8_t*)dblob;
    p.n_elem = n;
    p.next_elem = (int*)(dev + o_next);
    p.order = (const int32_t*)(dev + o_order);
    p.results = (DevResult*)(dev + o_res);
    p.max_z = (int32_t*)(dev + o_mz);
    p.post_z = (double*)(dev + o_pz);
    p.ws = dev + o_ws;
    p.ws_stride = ws1;
    p.n_int_max = n_int_max;
    p.GGp_max = GGp_max;
    p.stack_cap = c->stack_cap;
    p.counters = (DevCounters*)(dev + o_cnt);
    p.trial_burn = tb;
    p.trial_mcmc = tm;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ok = ok && cuda_ok(c, cudaEventCreate(&e0), "event") && cuda_ok(c, cudaEventCreate(&e1), "event");
    int best = -1;
    double best_rate = 0;
    float total_ms = 0;
    std::vector<DevResult> tres(n);
    for (int pass = 0; ok && pass < 2; pass++) {        // pass 0 warms every instance up on one element
        for (int i = 0; ok && i < (int)cand.size(); i++) {
            const ChainShape& s = cand[i];
            const int grid = std::max(1, std::min(n, c->n_sm * s.per_sm));
            p.n_elem = pass == 0 ? 1 : n;
            const size_t smem = smem_bytes(N, s.BT, prec, c->stack_cap);
            ok = cuda_ok(c, cudaMemsetAsync(dev + o_next, 0, 256, st), "memset (tuner)") &&
                 cuda_ok(c, cudaMemsetAsync(dev + o_res, 0, sizeof(DevResult) * n, st), "memset (tuner)") &&
                 cuda_ok(c, cudaEventRecord(e0, st), "event") &&
                 cuda_ok(c, launch_chain(p, grid, s.BT, smem, prec, s.variant, st), "launch (tuner)") &&
                 cuda_ok(c, cudaEventRecord(e1, st), "event") && cuda_ok(c, cudaEventSynchronize(e1), "tuner");
            float ms = 0;
            if (ok) cudaEventElapsedTime(&ms, e0, e1);
            total_ms += ms;
            if (ok && pass == 1) {
                ok = cuda_ok(c, cudaMemcpy(tres.data(), dev + o_res, sizeof(DevResult) * n, cudaMemcpyDeviceToHost),
                             "D2H (tuner)");
                double cyc = 0;
                for (int e = 0; e < n; e++) cyc += tres[e].device_ms;   // clock cycles of the element's chain
                const double rate = cyc > 0 ? (double)s.per_sm * n / cyc : 0;
                if (ok && (best < 0 || rate > best_rate)) { best = i; best_rate = rate; }
            }
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(dblob);
    cudaFree(dev);
    if (!ok || best < 0) return PACC_ECUDA;
    c->shape_trial_ms = total_ms;
    {
        std::lock_guard<std::mutex> lk(g_shape_mu);
        g_shape_cache[key] = {cand[best].variant, cand[best].BT};
    }
    return take(cand[best]);
}

// ---------------------------------------------------------------------------
// serving with the CTA-per-chain kernel (stream mode)
// ---------------------------------------------------------------------------
// Layout of one finished slot's results in the pinned staging (each part
// 16-byte aligned): result | Max_Z | P(Z) | rate traces | Z traces.
struct OutLayout {
    size_t mz, pz, trd, trz, bytes;
    OutLayout(const StreamServer& v, int N) {
        auto r16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
        mz = r16(sizeof(DevResult));
        pz = mz + r16(sizeof(int32_t) * 3 * N);
        trd = pz + r16(sizeof(double) * 3 * N * 4);
        trz = trd + r16(sizeof(double) * 3 * 6 * (size_t)v.TI);
        bytes = trz + r16((size_t)3 * v.TI * N);
    }
};
static size_t stream_out_bytes(const StreamServer& v, int N) { return OutLayout(v, N).bytes; }

static int stream_setup(pacc_ctx* c, int GG_needed, const std::vector<const HostElem*>& els) {
    StreamServer& v = c->ss;
    if (v.ready) return PACC_OK;
    cudaSetDevice(c->device);
    if (!ensure_model(c)) return PACC_ECUDA;
    const int N = c->M.N, S = c->M.S;
    const int T = c->o.burnin + c->o.mcmc;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    v.prec = c->o.precision == PACC_FP32 ? 1 : 0;
    v.GG_cap = std::max(5120, (GG_needed + 31) & ~31);
    v.GGp_cap = v.GG_cap;
    v.n_int_cap = S - 1;
    v.TI = std::min(c->o.trace_iters, T);
    const int sst = choose_shape(c, v.prec, els);
    if (sst != PACC_OK) return sst;
    v.BT = c->shape_bt;
    v.variant = c->shape_variant;
    v.smem = smem_bytes(N, v.BT, v.prec, c->stack_cap);
    const int per_sm = std::max(1, chain_occupancy(v.prec, v.variant, v.BT, v.smem));
    // one chain slot fewer than the GPU holds: the persistent launch fills
    // every SM's registers otherwise, and a small kernel of the same context
    // on another stream (pacc_pmatrix_noalloc) could not start until the
    // launch drained
    v.grid = std::max(1, c->n_sm * per_sm - 1);
    v.ws1 = (ws_bytes(v.n_int_cap, v.GGp_cap, T, c->o.mcmc, N, v.prec) + 4095) & ~(size_t)4095;
    const size_t tb = al(topo_bytes(N));
    v.o_tg = al((size_t)S * v.GGp_cap);
    v.o_prefix = al(v.o_tg + (size_t)v.n_int_cap * v.GGp_cap);
    v.o_topo = al(v.o_prefix + (size_t)(v.GGp_cap + 1) * 4);
    v.blob_b = al(v.o_topo + tb);
    const size_t per_slot = v.blob_b + sizeof(ElemHeader) + sizeof(DevResult) + 3 * N * 4 + 3 * N * 4 * 8 +
                            sizeof(double) * 3 * 6 * (size_t)v.TI + (size_t)3 * v.TI * N + 64;
    size_t budget = (size_t)c->o.memory_budget_bytes;
    if (budget == 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        budget = fr / 4;
    }
    const size_t fixed = v.ws1 * v.grid + (1 << 20);
    if (budget <= fixed + per_slot) { c->err = "memory budget too small for the serving workspaces"; return PACC_OOM; }
    // two queued chains per resident CTA keep every CTA busy between host polls
    const int want = c->o.max_resident > 0 ? c->o.max_resident : 2 * v.grid;
    v.n_slots = (int)std::min<size_t>((size_t)want, (budget - fixed) / per_slot);
    const int ns = v.n_slots;
    size_t o = 0;
    size_t o_hdr = o; o = al(o + sizeof(ElemHeader) * ns);
    size_t o_blob = o; o = al(o + v.blob_b * ns);
    size_t o_res = o; o = al(o + sizeof(DevResult) * ns);
    size_t o_mz = o; o = al(o + sizeof(int32_t) * 3 * N * (size_t)ns);
    size_t o_pz = o; o = al(o + sizeof(double) * 3 * N * 4 * (size_t)ns);
    size_t o_trd = o; o = al(o + sizeof(double) * 3 * 6 * (size_t)v.TI * ns);
    size_t o_trz = o; o = al(o + (size_t)3 * v.TI * N * ns);
    size_t o_cnt = o; o = al(o + sizeof(DevCounters));
    size_t o_head = o; o = al(o + 256);
    size_t o_ws = o; o = al(o + v.ws1 * v.grid);
    if (!cuda_ok(c, cudaMalloc((void**)&v.dev, o), "cudaMalloc (serving)")) return PACC_OOM;
    if (!cuda_ok(c, cudaMemset(v.dev, 0, o_ws), "memset")) return PACC_ECUDA;
    const size_t map_b = sizeof(int) * (64 + 2 * (size_t)ns);
    if (!cuda_ok(c, cudaHostAlloc((void**)&v.h_map, map_b, cudaHostAllocMapped), "cudaHostAlloc")) return PACC_OOM;
    std::memset(v.h_map, 0, map_b);
    int* d_map = nullptr;
    if (!cuda_ok(c, cudaHostGetDevicePointer((void**)&d_map, v.h_map, 0), "cudaHostGetDevicePointer"))
        return PACC_ECUDA;
    v.h_tail = v.h_map;
    v.h_stop = v.h_map + 1;
    v.h_qslot = v.h_map + 64;
    v.h_done = v.h_map + 64 + ns;
    // admission staging: at least four elements of the largest size
    v.h_stage_cap = std::max((size_t)32 << 20, 4 * (v.blob_b + sizeof(ElemHeader) + 64));
    if (!cuda_ok(c, cudaMallocHost((void**)&v.h_stage, v.h_stage_cap), "cudaMallocHost")) return PACC_OOM;
    v.out_chunk = (int)std::max<size_t>(1, std::min<size_t>(ns, ((size_t)16 << 20) / stream_out_bytes(v, N)));
    if (!cuda_ok(c, cudaMallocHost((void**)&v.h_out, stream_out_bytes(v, N) * v.out_chunk), "cudaMallocHost"))
        return PACC_OOM;
    if (!cuda_ok(c, cudaStreamCreateWithFlags(&v.copy, cudaStreamNonBlocking), "stream") ||
        !cuda_ok(c, cudaEventCreate(&v.ev0), "event") || !cuda_ok(c, cudaEventCreate(&v.ev1), "event"))
        return PACC_ECUDA;
    v.d_hdr = (ElemHeader*)(v.dev + o_hdr);
    v.d_blob = v.dev + o_blob;
    v.d_res = (DevResult*)(v.dev + o_res);
    v.d_mz = (int32_t*)(v.dev + o_mz);
    v.d_pz = (double*)(v.dev + o_pz);
    v.d_trd = v.TI > 0 ? (double*)(v.dev + o_trd) : nullptr;
    v.d_trz = v.TI > 0 ? (int8_t*)(v.dev + o_trz) : nullptr;
    v.d_cnt = (DevCounters*)(v.dev + o_cnt);
    v.d_head = (int*)(v.dev + o_head);
    v.d_ws = v.dev + o_ws;
    std::memset(&v.p, 0, sizeof(v.p));
    v.p.hdr = v.d_hdr;
    v.p.blob = (const uint8_t*)v.d_blob;
    v.p.n_elem = ns;
    v.p.results = v.d_res;
    v.p.max_z = v.d_mz;
    v.p.post_z = v.d_pz;
    v.p.tr_d = v.d_trd;
    v.p.tr_z = v.d_trz;
    v.p.ws = v.d_ws;
    v.p.ws_stride = v.ws1;
    v.p.n_int_max = v.n_int_cap;
    v.p.GGp_max = v.GGp_cap;
    v.p.stack_cap = c->stack_cap;
    v.p.counters = v.d_cnt;
    v.p.stream = 1;
    v.p.q_head = v.d_head;
    v.p.q_tail = d_map;
    v.p.q_slot = d_map + 64;
    v.p.q_cap = ns;
    v.p.done_flag = d_map + 64 + ns;
    v.p.q_stop = d_map + 1;
    // a safety bound: q_stop ends idle launches (default 30 s)
    v.p.idle_ns = c->o.serve_idle_ns > 0 ? (long long)c->o.serve_idle_ns : 30000000000LL;
    v.p.z_start_zero = c->o.chain > 0 ? 1 : 0;
    v.free_slots.clear();
    for (int i = ns - 1; i >= 0; i--) v.free_slots.push_back(i);
    v.busy.assign(ns, 0);
    v.slot_no.assign(ns, 0);
    v.slot_t0.assign(ns, 0);
    v.resident = 0;
    v.tail = 0;
    v.ready = true;
    return PACC_OK;
}

// Copies queued elements into free slots and publishes them to the queue.
static int stream_admit(pacc_ctx* c) {
    StreamServer& v = c->ss;
    const int N = c->M.N, S = c->M.S;
    std::vector<std::pair<int, std::pair<HostElem, double>>> adm;
    while (!v.free_slots.empty() && !v.queue.empty()) {
        int slot = v.free_slots.back();
        v.free_slots.pop_back();
        adm.push_back({slot, std::move(v.queue.front())});
        v.queue.pop_front();
    }
    if (adm.empty()) return PACC_OK;
    const size_t tb = topo_bytes(N);
    auto staged = [&](const HostElem& E) {
        return E.codes.size() + E.tg0.size() + E.prefix.size() * 4 + tb + sizeof(ElemHeader) + 64;
    };
    size_t off = 0;
    cudaStream_t st = v.copy;
    for (auto& a : adm) {
        const int slot = a.first;
        const HostElem& E = a.second.first;
        if (off + staged(E) > v.h_stage_cap) {
            // staging full: wait for its copies, then reuse it
            if (!cuda_ok(c, cudaStreamSynchronize(st), "admission")) return PACC_ECUDA;
            off = 0;
        }
        char* reg = v.d_blob + (size_t)slot * v.blob_b;
        ElemHeader H;
        std::memset(&H, 0, sizeof(H));
        H.GG = E.GG; H.GGp = E.GGp; H.root = E.root; H.n_nodes = E.n_nodes; H.n_int = E.n_int;
        H.n_hlev = E.n_hlev; H.n_dlev = E.n_dlev; H.tg_draws = E.tg_draws; H.stack_depth = E.stack_depth;
        H.element_no = E.no;
        H.SP = (S + 15) & ~15;
        H.codes_off = reg - v.d_blob;
        H.tg_off = H.codes_off + (int64_t)v.o_tg;
        H.prefix_off = H.codes_off + (int64_t)v.o_prefix;
        H.topo_off = H.codes_off + (int64_t)v.o_topo;
        char* p0 = v.h_stage + off;
        std::memcpy(p0, E.codes.data(), E.codes.size());
        char* p1 = p0 + E.codes.size();
        std::memcpy(p1, E.tg0.data(), E.tg0.size());
        char* p2 = p1 + E.tg0.size();
        std::memcpy(p2, E.prefix.data(), E.prefix.size() * 4);
        char* p3 = p2 + E.prefix.size() * 4;
        std::memcpy(p3, E.topo.data(), E.topo.size() * 2);
        std::memcpy(p3 + ((E.topo.size() * 2 + 15) & ~(size_t)15), E.dist2.data(), N * 8);
        char* p4 = p3 + tb;
        std::memcpy(p4, &H, sizeof(H));
        bool ok = cuda_ok(c, cudaMemcpyAsync(reg, p0, E.codes.size(), cudaMemcpyHostToDevice, st), "H2D codes") &&
                  cuda_ok(c, cudaMemcpyAsync(reg + v.o_tg, p1, E.tg0.size(), cudaMemcpyHostToDevice, st), "H2D tg") &&
                  cuda_ok(c, cudaMemcpyAsync(reg + v.o_prefix, p2, E.prefix.size() * 4, cudaMemcpyHostToDevice, st), "H2D prefix") &&
                  cuda_ok(c, cudaMemcpyAsync(reg + v.o_topo, p3, tb, cudaMemcpyHostToDevice, st), "H2D topo") &&
                  cuda_ok(c, cudaMemcpyAsync(v.d_hdr + slot, p4, sizeof(H), cudaMemcpyHostToDevice, st), "H2D header");
        // (no memset here: a memset is a kernel, which would wait for the
        // persistent launch to leave room on the SMs; the kernel writes every
        // result field of the slot before it raises the slot's flag)
        if (!ok) return PACC_ECUDA;
        off += staged(E);
        v.slot_no[slot] = E.no;
        v.slot_t0[slot] = a.second.second;
        v.busy[slot] = 1;
        v.resident++;
    }
    if (!cuda_ok(c, cudaStreamSynchronize(st), "admission")) return PACC_ECUDA;
    // the slots' data is in device memory: publish them
    for (auto& a : adm) {
        v.h_done[a.first] = 0;
        v.h_qslot[v.tail % v.n_slots] = a.first;
        v.tail++;
    }
    std::atomic_thread_fence(std::memory_order_seq_cst);
    *v.h_tail = v.tail;
    return PACC_OK;
}

// Collects the results of the slots whose chains finished.
static int stream_retire(pacc_ctx* c) {
    StreamServer& v = c->ss;
    const int N = c->M.N;
    std::vector<int> fin;
    for (int s = 0; s < v.n_slots; s++)
        if (v.busy[s] && v.h_done[s]) fin.push_back(s);
    if (fin.empty()) return PACC_OK;
    std::atomic_thread_fence(std::memory_order_seq_cst);
    const int nd = (int)fin.size();
    cudaStream_t st = v.copy;
    const size_t trd_n = (size_t)3 * 6 * v.TI, trz_n = (size_t)3 * v.TI * N;
    const OutLayout L(v, N);
    const size_t ob = L.bytes;
    int clk_khz = 0;
    cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, c->device);
    for (int i0 = 0; i0 < nd; i0 += v.out_chunk) {
        const int n = std::min(v.out_chunk, nd - i0);
        // per slot in the pinned staging: result | Max_Z | P(Z) | traces
        auto res_of = [&](int i) { return (DevResult*)(v.h_out + ob * i); };
        auto mz_of = [&](int i) { return (int32_t*)(v.h_out + ob * i + L.mz); };
        auto pz_of = [&](int i) { return (double*)(v.h_out + ob * i + L.pz); };
        auto trd_of = [&](int i) { return (double*)(v.h_out + ob * i + L.trd); };
        auto trz_of = [&](int i) { return (int8_t*)(v.h_out + ob * i + L.trz); };
        for (int i = 0; i < n; i++) {
            const int slot = fin[i0 + i];
            cudaMemcpyAsync(res_of(i), v.d_res + slot, sizeof(DevResult), cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(mz_of(i), v.d_mz + (size_t)slot * 3 * N, sizeof(int32_t) * 3 * N, cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(pz_of(i), v.d_pz + (size_t)slot * 3 * N * 4, sizeof(double) * 3 * N * 4,
                            cudaMemcpyDeviceToHost, st);
            if (v.TI > 0) {
                cudaMemcpyAsync(trd_of(i), v.d_trd + trd_n * slot, sizeof(double) * trd_n, cudaMemcpyDeviceToHost, st);
                cudaMemcpyAsync(trz_of(i), v.d_trz + trz_n * slot, trz_n, cudaMemcpyDeviceToHost, st);
            }
        }
        if (!cuda_ok(c, cudaStreamSynchronize(st), "D2H results")) return PACC_ECUDA;
        const double t = now_ms();
        for (int i = 0; i < n; i++) {
            const int slot = fin[i0 + i];
            pacc_ctx::Done d;
            std::memset(&d.r, 0, sizeof(d.r));
            d.r.element_no = v.slot_no[slot];
            d.r.n_nodes = N;
            const DevResult& R = *res_of(i);
            d.r.status = R.status == 0 ? PACC_OK : (R.status == 2 ? PACC_NAN_LIKELIHOOD : PACC_SAMPLER_ERROR);
            for (int m = 0; m < 3; m++) {
                pacc_model_result& mr = d.r.model[m];
                mr.loglik = R.model[m].loglik;
                mr.max_loglik = R.model[m].max_loglik;
                mr.n_rate = R.model[m].rates[0];
                mr.c_rate = R.model[m].rates[1];
                mr.g_rate = R.model[m].rates[2];
                mr.l_rate = R.model[m].rates[3];
                mr.l2_rate = R.model[m].rates[4];
                mr.failure = R.model[m].failure;
                mr.n_configs = R.model[m].n_configs;
            }
            d.r.device_ms = clk_khz > 0 ? R.device_ms / (double)clk_khz : 0.0;
            d.r.latency_ms = t - v.slot_t0[slot];
            d.max_z.assign(mz_of(i), mz_of(i) + 3 * N);
            d.post_z.assign(pz_of(i), pz_of(i) + 3 * N * 4);
            if (v.TI > 0) {
                d.tr_d.assign(trd_of(i), trd_of(i) + trd_n);
                d.tr_z.assign(trz_of(i), trz_of(i) + trz_n);
            }
            c->done.push_back(std::move(d));
            v.busy[slot] = 0;
            v.free_slots.push_back(slot);
            v.resident--;
        }
    }
    return PACC_OK;
}

// One host step of stream serving: collect finished chains, admit queued
// elements, and (re)launch the persistent kernel when chains wait and no
// launch is running.
static int stream_step(pacc_ctx* c) {
    StreamServer& v = c->ss;
    cudaSetDevice(c->device);
    int st = stream_retire(c);
    if (st != PACC_OK) return st;
    if (!ensure_model(c)) return PACC_ECUDA;
    st = stream_admit(c);
    if (st != PACC_OK) return st;
    if (v.running) {
        cudaError_t q = cudaEventQuery(v.ev1);
        if (q == cudaErrorNotReady && v.stopping && v.resident > 0) q = cudaEventSynchronize(v.ev1);
        if (q == cudaSuccess) {
            v.running = false;
            float ms = 0;
            cudaEventElapsedTime(&ms, v.ev0, v.ev1);
            v.kernel_ms += ms;
        } else if (q != cudaErrorNotReady) {
            return cuda_ok(c, q, "serving kernel") ? PACC_OK : PACC_ECUDA;
        }
    }
    // no chain left: let the idle blocks return (every block of a launch
    // stays until then, so a launch never runs on part of its blocks)
    if (v.running && v.resident == 0 && v.queue.empty() && !v.stopping) {
        *v.h_stop = 1;
        v.stopping = true;
    }
    if (!v.running && v.resident > 0) {
        *v.h_stop = 0;
        v.stopping = false;
        std::atomic_thread_fence(std::memory_order_seq_cst);
        cudaStream_t ks = c->stream;
        if (!cuda_ok(c, cudaEventRecord(v.ev0, ks), "event") ||
            !cuda_ok(c, launch_chain(v.p, v.grid, v.BT, v.smem, v.prec, v.variant, ks), "launch (serving)") ||
            !cuda_ok(c, cudaEventRecord(v.ev1, ks), "event"))
            return PACC_ECUDA;
        v.running = true;
        v.launches++;
    }
    return PACC_OK;
}

// Lets the queued and resident chains finish (their results go to done),
// then frees the serving slots, so that they can be made again for longer
// elements; launches, kernel time and device counters carry over.
static int stream_teardown(pacc_ctx* c) {
    StreamServer& v = c->ss;
    if (!v.ready) return PACC_OK;
    while (!v.queue.empty() || v.resident > 0) {
        const size_t nd = c->done.size();
        const int st = stream_step(c);
        if (st != PACC_OK) return st;
        if (c->done.size() == nd) std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
    int st = stream_step(c);   // asks the idle blocks to return
    if (st != PACC_OK) return st;
    if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "serving teardown")) return PACC_ECUDA;
    st = stream_step(c);       // accounts the ended launch's time
    if (st != PACC_OK) return st;
    DevCounters dc;
    if (!cuda_ok(c, cudaMemcpy(&dc, v.d_cnt, sizeof(dc), cudaMemcpyDeviceToHost), "serving teardown: counters"))
        return PACC_ECUDA;
    DevCounters carry = v.carry;
    carry.edge_internal += dc.edge_internal;
    carry.edge_leaf += dc.edge_leaf;
    carry.col_ll += dc.col_ll;
    carry.tg_draws += dc.tg_draws;
    carry.z_draws += dc.z_draws;
    carry.pmat += dc.pmat;
    carry.iters += dc.iters;
    for (int q = 0; q < 8; q++) carry.phase_cycles[q] += dc.phase_cycles[q];
    carry.idle_exits += dc.idle_exits;
    cudaFree(v.dev);
    cudaFreeHost(v.h_map);
    cudaFreeHost(v.h_stage);
    cudaFreeHost(v.h_out);
    cudaStreamDestroy(v.copy);
    cudaEventDestroy(v.ev0);
    cudaEventDestroy(v.ev1);
    const long long launches = v.launches;
    const double kernel_ms = v.kernel_ms;
    v = StreamServer();
    v.launches = launches;
    v.kernel_ms = kernel_ms;
    v.carry = carry;
    return PACC_OK;
}

int pacc_submit(pacc_ctx* c, const pacc_element_batch* b) {
    if (!c || !b || b->n_elements < 0) return PACC_EINVAL;
    const int n = b->n_elements;
    size_t base = c->pending.size();
    c->pending.resize(base + n);
    std::atomic<int> next(0);
    std::atomic<int> bad(0);
    int nt = std::max(1, std::min((int)std::thread::hardware_concurrency(), 32));
    if (n < 64) nt = 1;
    auto work = [&]() {
        for (;;) {
            int e = next.fetch_add(1);
            if (e >= n) break;
            HostElem& E = c->pending[base + e];
            E.no = b->element_no ? b->element_no[e] : e;
            if (b->lengths[e] < 0 || !preprocess(c->M, c->o, b->bases + b->offsets[e], b->lengths[e], E, false))
                bad = 1;
            // the chain kernels index an element's partials with 32-bit offsets
            else if ((size_t)8 * c->M.S * (size_t)E.GGp >= (size_t)INT32_MAX)
                bad = 1;
            // emission histogram bins are 16 bits; the prune's stack holds the full tree's depth
            else if (!E.filtered && (E.GG > 65535 || E.stack_depth > c->stack_cap))
                bad = 1;
            if (c->o.sample_hyper) {
                const int N = c->M.N;
                if (b->start_z) E.start_z.assign(b->start_z + (size_t)e * N, b->start_z + (size_t)(e + 1) * N);
                if (b->start_rates)
                    E.start_rates.assign(b->start_rates + (size_t)e * 5, b->start_rates + (size_t)(e + 1) * 5);
            }
        }
    };
    std::vector<std::thread> th;
    for (int i = 1; i < nt; i++) th.emplace_back(work);
    work();
    for (auto& t : th) t.join();
    if (bad) { c->pending.resize(base); c->err = "invalid element"; return PACC_EINVAL; }
    if (serving(c)) {
        if (!c->gpu_ok) return PACC_ECUDA;
        int gmax = 0;
        for (size_t i = base; i < c->pending.size(); i++) gmax = std::max(gmax, c->pending[i].GG);
        const bool warp = batched_layout(c);
        std::vector<const HostElem*> els;
        for (size_t i = base; i < c->pending.size(); i++) els.push_back(&c->pending[i]);
        if (!warp && c->ss.ready && gmax > c->ss.GG_cap) {
            // longer than the slots hold: the running chains finish under the
            // old set-up, then the slots are made for the new length
            const int st = stream_teardown(c);
            if (st != PACC_OK) { c->pending.resize(base); return st; }
        }
        int st = warp ? server_setup(c, gmax) : stream_setup(c, gmax, els);
        if (st != PACC_OK) { c->pending.resize(base); return st; }
        const int cap = warp ? c->srv.GG_cap : c->ss.GG_cap;
        auto& queue = warp ? c->srv.queue : c->ss.queue;
        const double t = now_ms();
        // within one submitted batch the longest elements are admitted first
        std::vector<size_t> ord;
        for (size_t i = base; i < c->pending.size(); i++) ord.push_back(i);
        std::stable_sort(ord.begin(), ord.end(),
                         [&](size_t a, size_t b) { return c->pending[a].GG > c->pending[b].GG; });
        for (size_t i : ord) {
            HostElem& E = c->pending[i];
            if (E.filtered) {
                pacc_ctx::Done d;
                std::memset(&d.r, 0, sizeof(d.r));
                d.r.element_no = E.no;
                d.r.n_nodes = c->M.N;
                d.r.status = E.filtered == 2 ? PACC_SAMPLER_ERROR : PACC_FILTERED;
                d.max_z.assign(3 * c->M.N, 0);
                d.post_z.assign(3 * c->M.N * 4, 0.0);
                c->done.push_back(std::move(d));
                continue;
            }
            if (E.GG > cap) {
                c->pending.resize(base);
                c->err = "element longer than the serving slot capacity";
                return PACC_EINVAL;
            }
            if (warp && (E.stack_depth > c->srv.D || E.n_int > c->srv.n_int_max)) {
                c->pending.resize(base);
                c->err = "element tree exceeds the serving slot geometry";
                return PACC_EUNSUPPORTED;
            }
            queue.push_back({std::move(E), t});
        }
        c->pending.resize(base);
    }
    return PACC_OK;
}

static void collect_results(pacc_ctx* c, const std::vector<DevResult>& res, const std::vector<int32_t>& mz,
                            const std::vector<double>& pz, const std::vector<double>& trd,
                            const std::vector<int8_t>& trz, int TI, int clk_khz,
                            const std::vector<int8_t>& ez, const std::vector<double>& er) {
    const int N = c->M.N;
    const int n = (int)c->pending.size();
    for (int e = 0; e < n; e++) {
        pacc_ctx::Done d;
        std::memset(&d.r, 0, sizeof(d.r));
        d.r.element_no = c->pending[e].no;
        d.r.n_nodes = N;
        HostElem& E = c->pending[e];
        if (E.filtered) {
            d.r.status = E.filtered == 2 ? PACC_SAMPLER_ERROR : PACC_FILTERED;
            d.max_z.assign(3 * N, 0);
            d.post_z.assign(3 * N * 4, 0.0);
        } else {
            const DevResult& R = res[e];
            d.r.status = R.status == 0 ? PACC_OK : (R.status == 2 ? PACC_NAN_LIKELIHOOD : PACC_SAMPLER_ERROR);
            for (int m = 0; m < 3; m++) {
                pacc_model_result& mr = d.r.model[m];
                mr.loglik = R.model[m].loglik;
                mr.max_loglik = R.model[m].max_loglik;
                mr.n_rate = R.model[m].rates[0];
                mr.c_rate = R.model[m].rates[1];
                mr.g_rate = R.model[m].rates[2];
                mr.l_rate = R.model[m].rates[3];
                mr.l2_rate = R.model[m].rates[4];
                mr.failure = R.model[m].failure;
                mr.n_configs = R.model[m].n_configs;
            }
            d.r.device_ms = clk_khz > 0 ? R.device_ms / (double)clk_khz : 0.0;
            d.max_z.assign(mz.begin() + (size_t)e * 3 * N, mz.begin() + (size_t)(e + 1) * 3 * N);
            d.post_z.assign(pz.begin() + (size_t)e * 3 * N * 4, pz.begin() + (size_t)(e + 1) * 3 * N * 4);
            if (TI > 0) {
                d.tr_d.assign(trd.begin() + (size_t)e * 3 * 6 * TI, trd.begin() + (size_t)(e + 1) * 3 * 6 * TI);
                d.tr_z.assign(trz.begin() + (size_t)e * 3 * TI * N, trz.begin() + (size_t)(e + 1) * 3 * TI * N);
            }
            if (!ez.empty()) {
                d.end_z.assign(ez.begin() + (size_t)e * N, ez.begin() + (size_t)(e + 1) * N);
                for (int q = 0; q < 5; q++) d.r.end_rates[q] = er[(size_t)e * 5 + q];
            }
        }
        c->done.push_back(std::move(d));
    }
}

static int run_batched(pacc_ctx* c, std::vector<ElemHeader>& hdr, std::vector<uint8_t>& blob, size_t off,
                       int n_int_max, int GGuP_max);

static int run_pending(pacc_ctx* c) {
    if (c->pending.empty()) return PACC_OK;
    if (!c->gpu_ok) return PACC_ECUDA;
    cudaSetDevice(c->device);
    if (!ensure_model(c)) return PACC_ECUDA;
    const int N = c->M.N, S = c->M.S;
    const int n = (int)c->pending.size();
    const int prec = c->o.precision == PACC_FP32 ? 1 : 0;
    const int T = c->o.burnin + c->o.mcmc;
    const int TI = std::min(c->o.trace_iters, T);
    // pack the blob
    std::vector<const HostElem*> els(n);
    for (int e = 0; e < n; e++) els[e] = &c->pending[e];
    std::vector<ElemHeader> hdr;
    std::vector<uint8_t> blob;
    int n_int_max, GGp_max, GGuP_max;
    const size_t off = pack_elems(c, els, hdr, blob, n_int_max, GGp_max, GGuP_max);
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    if (batched_layout(c)) return run_batched(c, hdr, blob, off, n_int_max, GGuP_max);
    // launch geometry: the context's shape (tuned at the first launch)
    const int sst = choose_shape(c, prec, els);
    if (sst != PACC_OK) return sst;
    const int BT = c->shape_bt, variant = c->shape_variant;
    size_t smem = smem_bytes(N, BT, prec, c->stack_cap);
    // resident CTAs per SM from the kernel's registers and shared memory
    int per_sm = std::max(1, chain_occupancy(prec, variant, BT, smem));
    int grid = std::max(1, std::min(n, c->n_sm * per_sm));
    size_t ws1 = ws_bytes(n_int_max, GGp_max, T, c->o.mcmc, N, prec);
    ws1 = (ws1 + 4095) & ~(size_t)4095;
    // misc buffers
    size_t o_hdr = 0;
    size_t o_res = al(o_hdr + sizeof(ElemHeader) * n);
    size_t o_mz = al(o_res + sizeof(DevResult) * n);
    size_t o_pz = al(o_mz + sizeof(int32_t) * 3 * N * (size_t)n);
    size_t o_trd = al(o_pz + sizeof(double) * 3 * N * 4 * (size_t)n);
    size_t o_trz = al(o_trd + sizeof(double) * 3 * 6 * (size_t)TI * n);
    size_t o_cnt = al(o_trz + (size_t)3 * TI * N * n);
    size_t o_next = al(o_cnt + sizeof(DevCounters));
    size_t o_order = al(o_next + 256);
    // SAMPLE_HYPER: start and end states
    const bool hyp = c->o.sample_hyper != 0;
    size_t o_sz = al(o_order + sizeof(int32_t) * n);
    size_t o_sr = al(o_sz + (hyp ? (size_t)N * n : 0));
    size_t o_ez = al(o_sr + (hyp ? sizeof(double) * 5 * n : 0));
    size_t o_er = al(o_ez + (hyp ? (size_t)N * n : 0));
    size_t misc = al(o_er + (hyp ? sizeof(double) * 5 * n : 0));
    if (!grow(c, &c->d_blob, &c->blob_cap, std::max<size_t>(off, 256)) ||
        !grow(c, &c->d_ws, &c->ws_cap, ws1 * grid) || !grow(c, &c->d_misc, &c->misc_cap, misc))
        return PACC_OOM;
    // CTAs claim the longest elements first, so that the last chains to start are short
    std::vector<int32_t> order(n);
    for (int e = 0; e < n; e++) order[e] = e;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return c->pending[a].GG > c->pending[b].GG; });
    char* mb = (char*)c->d_misc;
    cudaStream_t st = c->stream;
    if (!cuda_ok(c, cudaMemcpyAsync(c->d_blob, blob.data(), off, cudaMemcpyHostToDevice, st), "H2D blob") ||
        !cuda_ok(c, cudaMemcpyAsync(mb + o_hdr, hdr.data(), sizeof(ElemHeader) * n, cudaMemcpyHostToDevice, st),
                 "H2D hdr") ||
        !cuda_ok(c, cudaMemsetAsync(mb + o_res, 0, o_next + 256 - o_res, st), "memset") ||
        !cuda_ok(c, cudaMemcpyAsync(mb + o_order, order.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st),
                 "H2D order"))
        return PACC_ECUDA;
    std::vector<int8_t> sz, ez;
    std::vector<double> sr, er;
    if (hyp) {
        // start states: the caller's, else the first chain's (Z marked -128,
        // rates from INIT_*, main.cpp:286 for l2)
        sz.assign((size_t)N * n, 0);
        sr.assign((size_t)5 * n, 0.0);
        for (int e = 0; e < n; e++) {
            const HostElem& E = c->pending[e];
            if ((int)E.start_z.size() == N) std::memcpy(&sz[(size_t)e * N], E.start_z.data(), N);
            else sz[(size_t)e * N] = -128;
            if (E.start_rates.size() == 5) {
                for (int q = 0; q < 5; q++) sr[(size_t)e * 5 + q] = E.start_rates[q];
            } else {
                const pacc_opts& o = c->o;
                const double l2 = (o.hyper_lrate2_a == 0) ? 0.0 : o.init_lrate2;
                const double v[5] = {o.init_acce_rate, o.init_conserve_rate, o.init_grate, o.init_lrate, l2};
                for (int q = 0; q < 5; q++) sr[(size_t)e * 5 + q] = v[q];
            }
        }
        ez.assign((size_t)N * n, 0);
        er.assign((size_t)5 * n, 0.0);
        if (!cuda_ok(c, cudaMemcpyAsync(mb + o_sz, sz.data(), sz.size(), cudaMemcpyHostToDevice, st), "H2D start Z") ||
            !cuda_ok(c, cudaMemcpyAsync(mb + o_sr, sr.data(), sr.size() * 8, cudaMemcpyHostToDevice, st),
                     "H2D start rates"))
            return PACC_ECUDA;
    }
    ChainParams p;
    std::memset(&p, 0, sizeof(p));
    p.hdr = (const ElemHeader*)(mb + o_hdr);
    p.blob = (const uint8_t*)c->d_blob;
    p.n_elem = n;
    p.next_elem = (int*)(mb + o_next);
    p.order = (const int32_t*)(mb + o_order);
    p.results = (DevResult*)(mb + o_res);
    p.max_z = (int32_t*)(mb + o_mz);
    p.post_z = (double*)(mb + o_pz);
    p.tr_d = TI > 0 ? (double*)(mb + o_trd) : nullptr;
    p.tr_z = TI > 0 ? (int8_t*)(mb + o_trz) : nullptr;
    p.ws = (char*)c->d_ws;
    p.ws_stride = ws1;
    p.n_int_max = n_int_max;
    p.GGp_max = GGp_max;
    p.stack_cap = c->stack_cap;
    p.counters = (DevCounters*)(mb + o_cnt);
    p.z_start_zero = c->o.chain > 0 ? 1 : 0;
    if (hyp) {
        p.first_model = 2;
        p.start_z = (const int8_t*)(mb + o_sz);
        p.start_rates = (const double*)(mb + o_sr);
        p.end_z = (int8_t*)(mb + o_ez);
        p.end_rates = (double*)(mb + o_er);
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    if (!cuda_ok(c, launch_chain(p, grid, BT, smem, prec, variant, st), "launch chain")) return PACC_ECUDA;
    cudaEventRecord(e1, st);
    std::vector<DevResult> res(n);
    std::vector<int32_t> mz((size_t)3 * N * n);
    std::vector<double> pz((size_t)3 * N * 4 * n);
    std::vector<double> trd((size_t)3 * 6 * TI * n);
    std::vector<int8_t> trz((size_t)3 * TI * N * n);
    DevCounters dc;
    cudaMemcpyAsync(res.data(), mb + o_res, sizeof(DevResult) * n, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(mz.data(), mb + o_mz, mz.size() * 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(pz.data(), mb + o_pz, pz.size() * 8, cudaMemcpyDeviceToHost, st);
    if (TI > 0) {
        cudaMemcpyAsync(trd.data(), mb + o_trd, trd.size() * 8, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(trz.data(), mb + o_trz, trz.size(), cudaMemcpyDeviceToHost, st);
    }
    cudaMemcpyAsync(&dc, mb + o_cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, st);
    if (hyp) {
        cudaMemcpyAsync(ez.data(), mb + o_ez, ez.size(), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(er.data(), mb + o_er, er.size() * 8, cudaMemcpyDeviceToHost, st);
    }
    if (!cuda_ok(c, cudaStreamSynchronize(st), "chain kernel")) return PACC_ECUDA;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int clk_khz = 0;
    cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, c->device);
    pacc_counters& pc = c->counters;
    std::memset(&pc, 0, sizeof(pc));
    pc.edge_updates_internal = (double)dc.edge_internal;
    pc.edge_updates_leaf = (double)dc.edge_leaf;
    pc.column_loglik = (double)dc.col_ll;
    pc.tg_draws = (double)dc.tg_draws;
    pc.z_draws = (double)dc.z_draws;
    pc.pmatrix_builds = (double)dc.pmat;
    pc.iterations = (double)dc.iters;
    for (int q = 0; q < 8; q++) pc.phase_cycles[q] = (double)dc.phase_cycles[q];
    pc.kernel_ms = ms;
    pc.flop = 36.0 * pc.edge_updates_internal + 4.0 * pc.edge_updates_leaf;
    collect_results(c, res, mz, pz, trd, trz, TI, clk_khz, ez, er);
    c->pending.clear();
    (void)S;
    return PACC_OK;
}


// The batched path: one warp per element chain, chain state resident in device
// memory (pacc_batch.cu).  Every admitted element gets a slot; warps claim
// slots from a queue and run each chain to completion.
static int run_batched(pacc_ctx* c, std::vector<ElemHeader>& hdr, std::vector<uint8_t>& blob, size_t off,
                       int n_int_max, int GGuP_max) {
    const int N = c->M.N, S = c->M.S;
    const int n = (int)c->pending.size();
    const int prec = c->o.precision == PACC_FP32_WARP ? 1 : 0;
    const int T = c->o.burnin + c->o.mcmc;
    const int TI = std::min(c->o.trace_iters, T);
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    std::vector<int32_t> elem;
    for (int e = 0; e < n; e++) if (!c->pending[e].filtered) elem.push_back(e);
    // longest elements first: the last chains to start are the short ones
    std::stable_sort(elem.begin(), elem.end(),
                     [&](int a, int b) { return c->pending[a].GG > c->pending[b].GG; });
    const int n_slots = std::max(1, (int)elem.size());
    if (elem.empty()) elem.push_back(-1);
    int D = 1;
    for (int e = 0; e < n; e++) if (!c->pending[e].filtered) D = std::max(D, c->pending[e].stack_depth);
    // geometry per column count; the column count itself is tuned (or the caller's)
    {
        std::vector<int> cands = batch_candidates(c, prec);
        size_t grp_max = 0;
        int warps_max = 0;
        for (int Cc : cands) {
            BatchGeom g;
            if (!batch_geom(c, prec, Cc, n_int_max, D, n_slots, GGuP_max, g)) continue;
            grp_max = std::max(grp_max, g.grp_b);
            warps_max = std::max(warps_max, g.grid * g.warps);
        }
        if (warps_max == 0) { c->err = "element tree too large for the batched kernel"; return PACC_EUNSUPPORTED; }
        c->tune_grp_b = grp_max;
        c->tune_warps = warps_max;
    }
    const size_t grp_b = c->tune_grp_b;
    const int n_warps = c->tune_warps;
    size_t slot_b = al(batch_slot_bytes(N, T));
    size_t o_hdr = 0;
    size_t o_res = al(o_hdr + sizeof(ElemHeader) * n);
    size_t o_mz = al(o_res + sizeof(DevResult) * n);
    size_t o_pz = al(o_mz + sizeof(int32_t) * 3 * N * (size_t)n);
    size_t o_trd = al(o_pz + sizeof(double) * 3 * N * 4 * (size_t)n);
    size_t o_trz = al(o_trd + sizeof(double) * 3 * 6 * (size_t)TI * n);
    size_t o_cnt = al(o_trz + (size_t)3 * TI * N * n);
    size_t o_next = al(o_cnt + sizeof(DevCounters));
    size_t o_elem = al(o_next + 256);
    size_t o_slots = al(o_elem + sizeof(int32_t) * elem.size());
    size_t o_slotws = al(o_slots + sizeof(SlotState) * n_slots);
    size_t o_grp = al(o_slotws + slot_b * n_slots);
    size_t misc = al(o_grp + grp_b * n_warps);
    if (!grow(c, &c->d_blob, &c->blob_cap, std::max<size_t>(off, 256)) || !grow(c, &c->d_misc, &c->misc_cap, misc))
        return PACC_OOM;
    char* mb = (char*)c->d_misc;
    cudaStream_t st = c->stream;
    if (!cuda_ok(c, cudaMemcpyAsync(c->d_blob, blob.data(), off, cudaMemcpyHostToDevice, st), "H2D blob") ||
        !cuda_ok(c, cudaMemcpyAsync(mb + o_hdr, hdr.data(), sizeof(ElemHeader) * n, cudaMemcpyHostToDevice, st), "H2D hdr"))
        return PACC_ECUDA;
    BatchParams p;
    std::memset(&p, 0, sizeof(p));
    p.hdr = (const ElemHeader*)(mb + o_hdr);
    p.blob = (const uint8_t*)c->d_blob;
    p.slots = (SlotState*)(mb + o_slots);
    p.n_slots = n_slots;
    p.slot_ws = mb + o_slotws;
    p.slot_ws_stride = slot_b;
    p.grp_ws = mb + o_grp;
    p.grp_ws_stride = grp_b;
    p.sweeps = c->o.sweeps_per_launch;
    p.results = (DevResult*)(mb + o_res);
    p.max_z = (int32_t*)(mb + o_mz);
    p.post_z = (double*)(mb + o_pz);
    p.tr_d = TI > 0 ? (double*)(mb + o_trd) : nullptr;
    p.tr_z = TI > 0 ? (int8_t*)(mb + o_trz) : nullptr;
    p.counters = (DevCounters*)(mb + o_cnt);
    p.n_done = (int*)(mb + o_next);
    p.next_slot = (int*)(mb + o_next + 128);
    p.n_int_max = n_int_max;
    p.S_max = S;
    p.stack_depth = D;
    p.GGuP_max = GGuP_max;
    // column count: the caller's, the tuned one for this tree and precision,
    // or tuned now on a sample of this batch
    int C = 0;
    {
        int st_t = tune_columns(c, prec, D, n_int_max, GGuP_max, elem, p, mb + o_elem, mb + o_next, C);
        if (st_t != PACC_OK) return st_t;
    }
    BatchGeom g;
    batch_geom(c, prec, C, n_int_max, D, n_slots, GGuP_max, g);
    const int warps = g.warps, grid = g.grid;
    const size_t smem = g.smem;
    if (!cuda_ok(c, cudaMemcpyAsync(mb + o_elem, elem.data(), sizeof(int32_t) * elem.size(), cudaMemcpyHostToDevice, st), "H2D elem") ||
        !cuda_ok(c, cudaMemsetAsync(mb + o_res, 0, o_elem - o_res, st), "memset") ||
        !cuda_ok(c, launch_init_slots(mb + o_slots, (const int32_t*)(mb + o_elem), n_slots, st), "init slots"))
        return PACC_ECUDA;
    p.n_slots = n_slots;
    p.sweeps = c->o.sweeps_per_launch;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    int launches = 0;
    for (;;) {
        if (!cuda_ok(c, cudaMemsetAsync(mb + o_next + 128, 0, 4, st), "memset queue") ||
            !cuda_ok(c, launch_batch(&p, grid, warps, smem, prec, C, st), "launch batch"))
            return PACC_ECUDA;
        launches++;
        if (p.sweeps <= 0) break;
        int done = 0;
        if (!cuda_ok(c, cudaMemcpyAsync(&done, mb + o_next, 4, cudaMemcpyDeviceToHost, st), "D2H done") ||
            !cuda_ok(c, cudaStreamSynchronize(st), "batch kernel"))
            return PACC_ECUDA;
        if (done >= (int)elem.size() || elem[0] < 0) break;
        if (launches > 100000000) { c->err = "batched run did not finish"; return PACC_TIMEOUT; }
    }
    cudaEventRecord(e1, st);
    std::vector<DevResult> res(n);
    std::vector<int32_t> mz((size_t)3 * N * n);
    std::vector<double> pz((size_t)3 * N * 4 * n);
    std::vector<double> trd((size_t)3 * 6 * TI * n);
    std::vector<int8_t> trz((size_t)3 * TI * N * n);
    DevCounters dc;
    cudaMemcpyAsync(res.data(), mb + o_res, sizeof(DevResult) * n, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(mz.data(), mb + o_mz, mz.size() * 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(pz.data(), mb + o_pz, pz.size() * 8, cudaMemcpyDeviceToHost, st);
    if (TI > 0) {
        cudaMemcpyAsync(trd.data(), mb + o_trd, trd.size() * 8, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(trz.data(), mb + o_trz, trz.size(), cudaMemcpyDeviceToHost, st);
    }
    cudaMemcpyAsync(&dc, mb + o_cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, st);
    if (!cuda_ok(c, cudaStreamSynchronize(st), "batch kernel")) return PACC_ECUDA;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int clk_khz = 0;
    cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, c->device);
    pacc_counters& pc = c->counters;
    std::memset(&pc, 0, sizeof(pc));
    pc.edge_updates_internal = (double)dc.edge_internal;
    pc.edge_updates_leaf = (double)dc.edge_leaf;
    pc.tg_draws = (double)dc.tg_draws;
    pc.kernel_ms = ms;
    pc.flop = 36.0 * pc.edge_updates_internal + 4.0 * pc.edge_updates_leaf;
    pc.iterations = (double)launches;
    for (int q = 0; q < 8; q++) pc.phase_cycles[q] = (double)dc.phase_cycles[q];
    collect_results(c, res, mz, pz, trd, trz, TI, clk_khz, {}, {});
    c->pending.clear();
    return PACC_OK;
}

int pacc_sync(pacc_ctx* c) {
    if (!c) return PACC_EINVAL;
    if (serving(c)) {
        if (batched_layout(c)) {
            while (!c->srv.queue.empty() || c->srv.resident > 0 || c->srv.inflight) {
                int st = server_step(c);
                if (st != PACC_OK) return st;
            }
        } else {
            while (!c->ss.queue.empty() || c->ss.resident > 0) {
                const size_t nd = c->done.size();
                int st = stream_step(c);
                if (st != PACC_OK) return st;
                if (c->done.size() == nd) std::this_thread::sleep_for(std::chrono::microseconds(200));
            }
            int st = stream_step(c);   // asks the idle blocks to return
            if (st != PACC_OK) return st;
        }
        return PACC_OK;
    }
    return run_pending(c);
}

int pacc_pending(pacc_ctx* c) {
    if (!c) return 0;
    return (int)(c->pending.size() + c->srv.queue.size() + c->srv.resident + c->ss.queue.size() + c->ss.resident +
                 (c->done.size() - c->done_head));
}

static void fill_result(pacc_ctx* c, pacc_ctx::Done& d, pacc_result* out) {
    const int N = c->M.N;
    int32_t* mz = out->max_z;
    double* pz = out->post_z;
    pacc_trace tr = out->trace;
    int8_t* ez = out->end_z;
    *out = d.r;
    out->max_z = mz;
    out->post_z = pz;
    out->trace = tr;
    out->end_z = ez;
    if (ez && !d.end_z.empty()) std::memcpy(ez, d.end_z.data(), (size_t)N);
    if (mz) std::memcpy(mz, d.max_z.data(), sizeof(int32_t) * 3 * N);
    if (pz) std::memcpy(pz, d.post_z.data(), sizeof(double) * 3 * N * 4);
    const int T = c->o.burnin + c->o.mcmc;
    const int TI = std::min(c->o.trace_iters, T);
    const int TS = c->o.trace_iters;  // caller stride
    if (TI > 0 && !d.tr_d.empty()) {
        double* dst[6] = {tr.loglik, tr.n_rate, tr.c_rate, tr.g_rate, tr.l_rate, tr.l2_rate};
        for (int m = 0; m < 3; m++)
            for (int r = 0; r < 6; r++)
                if (dst[r])
                    for (int i = 0; i < TI; i++) dst[r][m * TS + i] = d.tr_d[((size_t)m * 6 + r) * TI + i];
        if (tr.z)
            for (int m = 0; m < 3; m++)
                for (int i = 0; i < TI; i++)
                    for (int s = 0; s < N; s++)
                        tr.z[((size_t)m * TS + i) * N + s] = d.tr_z[((size_t)m * TI + i) * N + s];
    }
}

int pacc_poll(pacc_ctx* c, pacc_result* out, int max) {
    if (!c || (!out && max > 0)) return -PACC_EINVAL;
    if (serving(c) && c->done_head == c->done.size()) {
        if (batched_layout(c)) {
            if (!c->srv.queue.empty() || c->srv.resident > 0 || c->srv.inflight) {
                int st = server_step(c);
                if (st != PACC_OK) return -st;
            }
        } else if (!c->ss.queue.empty() || c->ss.resident > 0) {
            int st = stream_step(c);
            if (st != PACC_OK) return -st;
            if (c->done_head == c->done.size()) {   // nothing finished yet: do not spin the caller
                std::this_thread::sleep_for(std::chrono::microseconds(200));
                st = stream_step(c);
                if (st != PACC_OK) return -st;
            }
        }
    }
    int k = 0;
    while (k < max && c->done_head < c->done.size()) {
        fill_result(c, c->done[c->done_head], &out[k]);
        c->done_head++;
        k++;
    }
    if (c->done_head == c->done.size()) { c->done.clear(); c->done_head = 0; }
    return k;
}

int pacc_run(pacc_ctx* c, const pacc_element_batch* b, pacc_result* out) {
    if (!c || !b) return PACC_EINVAL;
    if (!c->pending.empty() || c->done_head < c->done.size()) { c->err = "pacc_run needs an idle context"; return PACC_EBUSY; }
    int st = pacc_submit(c, b);
    if (st != PACC_OK) return st;
    st = pacc_sync(c);
    if (st != PACC_OK) return st;
    if (serving(c)) {
        // results arrive in completion order: put them back in batch order
        std::unordered_map<int64_t, std::deque<int>> where;
        for (int i = 0; i < b->n_elements; i++) where[b->element_no ? b->element_no[i] : i].push_back(i);
        const size_t n0 = c->done_head;
        if (c->done.size() - n0 != (size_t)b->n_elements) { c->err = "served results lost"; return PACC_ECUDA; }
        std::vector<pacc_ctx::Done> ord(b->n_elements);
        for (size_t j = n0; j < c->done.size(); j++) {
            auto it = where.find(c->done[j].r.element_no);
            if (it == where.end() || it->second.empty()) { c->err = "served results lost"; return PACC_ECUDA; }
            ord[it->second.front()] = std::move(c->done[j]);
            it->second.pop_front();
        }
        for (int i = 0; i < b->n_elements; i++) c->done[n0 + i] = std::move(ord[i]);
    }
    int k = pacc_poll(c, out, b->n_elements);
    return k == b->n_elements ? PACC_OK : PACC_ECUDA;
}

int pacc_get_counters(pacc_ctx* c, pacc_counters* out) {
    if (!c || !out) return PACC_EINVAL;
    if (serving(c) && !batched_layout(c) && c->ss.ready) {
        DevCounters dc;
        if (cudaMemcpyAsync(&dc, c->ss.d_cnt, sizeof(dc), cudaMemcpyDeviceToHost, c->ss.copy) != cudaSuccess ||
            cudaStreamSynchronize(c->ss.copy) != cudaSuccess)
            return PACC_ECUDA;
        pacc_counters& pc = c->counters;
        std::memset(&pc, 0, sizeof(pc));
        const DevCounters& cy = c->ss.carry;
        pc.edge_updates_internal = (double)(dc.edge_internal + cy.edge_internal);
        pc.edge_updates_leaf = (double)(dc.edge_leaf + cy.edge_leaf);
        pc.column_loglik = (double)(dc.col_ll + cy.col_ll);
        pc.tg_draws = (double)(dc.tg_draws + cy.tg_draws);
        pc.z_draws = (double)(dc.z_draws + cy.z_draws);
        pc.pmatrix_builds = (double)(dc.pmat + cy.pmat);
        double running_ms = 0;
        if (c->ss.running && cudaEventQuery(c->ss.ev0) == cudaSuccess) {
            // the launch in progress: time from its start event to now
            cudaEvent_t now;
            cudaEventCreate(&now);
            cudaEventRecord(now, c->ss.copy);
            cudaEventSynchronize(now);
            float ms = 0;
            cudaEventElapsedTime(&ms, c->ss.ev0, now);
            cudaEventDestroy(now);
            running_ms = ms;
        }
        for (int q = 0; q < 8; q++) pc.phase_cycles[q] = (double)(dc.phase_cycles[q] + cy.phase_cycles[q]);
        pc.kernel_ms = c->ss.kernel_ms + running_ms;
        pc.flop = 36.0 * pc.edge_updates_internal + 4.0 * pc.edge_updates_leaf;
        pc.iterations = (double)c->ss.launches;
        pc.serve_idle_exits = (double)(dc.idle_exits + cy.idle_exits);
    } else if (serving(c) && c->srv.ready) {
        if (c->srv.inflight) cudaStreamSynchronize(c->stream);
        DevCounters dc;
        if (cudaMemcpy(&dc, c->srv.d_cnt, sizeof(dc), cudaMemcpyDeviceToHost) != cudaSuccess) return PACC_ECUDA;
        pacc_counters& pc = c->counters;
        std::memset(&pc, 0, sizeof(pc));
        pc.edge_updates_internal = (double)dc.edge_internal;
        pc.edge_updates_leaf = (double)dc.edge_leaf;
        pc.tg_draws = (double)dc.tg_draws;
        pc.kernel_ms = c->srv.kernel_ms;
        pc.flop = 36.0 * pc.edge_updates_internal + 4.0 * pc.edge_updates_leaf;
        pc.iterations = (double)c->srv.steps;
        for (int q = 0; q < 8; q++) pc.phase_cycles[q] = (double)dc.phase_cycles[q];
    }
    *out = c->counters;
    return PACC_OK;
}

int pacc_get_launch_shape(pacc_ctx* c, int32_t* block_threads, int32_t* registers, int32_t* chains_per_sm,
                          double* trial_ms) {
    if (!c) return PACC_EINVAL;
    const bool cta = !batched_layout(c) && c->shape_ready;
    const int prec = c->o.precision == PACC_FP32 ? 1 : 0;
    if (block_threads) *block_threads = cta ? c->shape_bt : 0;
    if (registers) *registers = cta ? chain_regs(prec, c->shape_variant) : 0;
    if (chains_per_sm) *chains_per_sm = cta ? c->shape_per_sm : 0;
    if (trial_ms) *trial_ms = cta ? c->shape_trial_ms : 0;
    return PACC_OK;
}


void pacc_gbgc_default_opts(pacc_gbgc_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->burnin = 200; o->mcmc = 800; o->seed = 7728; o->gapchar = '*';
    o->conserve_rate = -2.0; o->acce_rate = 0.0; o->init_gc = 3.0;
    o->conserve_prior_a = 5.0; o->conserve_prior_b = 0.4;
    o->acce_prior_a = 5.0; o->acce_prior_b = 0.4; o->acce_prior_shift = 2.0;
    o->gc_prior_a = 4.0; o->gc_prior_b = 0.8; o->gc_prior_c = 0.2;
    o->prep_lrate = 0.1; o->prep_grate = 0.8;
    o->cons_to_mis = 0.01; o->ncons_to_mis = 0.1;
    o->missing_thres = 0.8; o->conserve_prop = 0.8;
    o->prop_c = 1.2; o->prop_n = 1.2; o->prop_gc = 0.2;
}


int pacc_gbgc_sync(pacc_ctx* c) {
    if (!c) return PACC_EINVAL;
    GbgcServer& v = c->gs;
    if (!v.ready) return PACC_OK;
    cudaSetDevice(c->device);
    while (v.resident > 0 || !v.queue.empty()) {
        int st = gbgc_collect(c);
        if (st == PACC_OK) st = gbgc_pump(c);
        if (st != PACC_OK) return st;
        if (v.running) {
            const cudaError_t e = cudaEventQuery(v.ev_done);
            if (e != cudaSuccess && e != cudaErrorNotReady) return cuda_ok(c, e, "gbgc serving launch") ? PACC_OK : PACC_ECUDA;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
    // nothing left: the blocks return now, and the launch's time and phase
    // cycles are counted
    if (v.running) {
        *v.h_stop = 1;
        float ms = 0;
        if (!cuda_ok(c, cudaEventSynchronize(v.ev_done), "gbgc serving launch")) return PACC_ECUDA;
        if (cudaEventElapsedTime(&ms, v.ev0, v.ev_done) == cudaSuccess) c->counters.kernel_ms += ms;
        v.running = false;
        unsigned long long ph[8], fl = 0;
        if (cuda_ok(c, cudaMemcpy(ph, v.p.phase, sizeof(ph), cudaMemcpyDeviceToHost), "D2H (phases)") &&
            cuda_ok(c, cudaMemcpy(&fl, v.p.flop, sizeof(fl), cudaMemcpyDeviceToHost), "D2H (flop)") &&
            cuda_ok(c, cudaMemset(v.p.phase, 0, sizeof(ph)), "memset (phases)") &&
            cuda_ok(c, cudaMemset(v.p.flop, 0, sizeof(fl)), "memset (flop)")) {
            for (int q = 0; q < 8; q++) c->counters.phase_cycles[q] += (double)ph[q];
            c->counters.flop += (double)fl;
        }
    }
    return PACC_OK;
}

int pacc_gbgc_submit(pacc_ctx* c, const pacc_gbgc_opts* go, const pacc_element_batch* b) {
    if (!c) return PACC_EINVAL;
    if (!go || !b || b->n_elements < 0 || (b->n_elements > 0 && (!b->lengths || !b->offsets || !b->bases))) {
        c->err = "gbgc_submit: options and batch must be non-null";
        return PACC_EINVAL;
    }
    if (go->burnin < 0 || go->mcmc < 2 || go->prop_c <= 1 || go->prop_n <= 1 || go->prop_gc <= 0) {
        c->err = "gbgc_submit: burnin >= 0, mcmc >= 2, prop_c and prop_n > 1, prop_gc > 0";
        return PACC_EINVAL;
    }
    if (!c->gpu_ok) { c->err = "gbgc_submit: no usable GPU"; return PACC_ECUDA; }
    cudaSetDevice(c->device);
    GbgcServer& v = c->gs;
    const HostModel& M = c->M;
    const int n = b->n_elements;
    const double t0 = gbgc_now();
    std::vector<GbgcServer::Pending> pend(n);
    {
        const int nth = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
        std::atomic<int> next(0);
        std::vector<std::thread> th;
        for (int t = 0; t < nth; t++)
            th.emplace_back([&]() {
                for (int i = next++; i < n; i = next++) {
                    GbgcServer::Pending& q = pend[i];
                    gbgc_prepare(M, b->bases + b->offsets[i], b->lengths[i], (char)go->gapchar, go->missing_thres,
                                 go->conserve_prop, q.E);
                    if (!q.E.filtered) {
                        int nint = 0;
                        for (int s2 : q.E.nodes) nint += s2 >= M.S;
                        if (nint == 0) q.E.filtered = 2;
                    }
                    if (!q.E.filtered) gbgc_blob(M, q.E, q.H, q.blob);
                    q.no = b->element_no ? b->element_no[i] : i;
                    q.t0 = t0;
                    q.filtered = q.E.filtered;
                }
            });
        for (auto& t : th) t.join();
    }
    int GGp_need = 32;
    for (auto& q : pend)
        if (!q.filtered) GGp_need = std::max(GGp_need, q.E.GGp);
    const int prec = (c->o.precision == PACC_FP32 || c->o.precision == PACC_FP32_WARP) ? 1 : 0;
    if (v.ready && (!gbgc_same_opts(*go, v) || GGp_need > v.GGp_cap || prec != v.prec)) {
        const int st = pacc_gbgc_sync(c);   // the running elements finish under the old set-up
        if (st != PACC_OK) return st;
        gbgc_serve_teardown(c);
    }
    if (!v.ready) {
        const int st = gbgc_serve_setup(c, *go, GGp_need);
        if (st != PACC_OK) return st;
    }
    for (auto& q : pend) {
        if (q.filtered) {
            GbgcServer::Done d;
            std::memset(&d.r, 0, sizeof(d.r));
            d.r.element_no = q.no;
            d.r.status = PACC_FILTERED;
            d.r.root = -1;
            v.done.push_back(std::move(d));
        } else {
            v.queue.push_back(std::move(q));
        }
    }
    return gbgc_pump(c);
}

int pacc_gbgc_poll(pacc_ctx* c, pacc_gbgc_result* out, int max) {
    if (!c || (max > 0 && !out)) return PACC_EINVAL;
    GbgcServer& v = c->gs;
    if (v.ready) {
        cudaSetDevice(c->device);
        int st = gbgc_collect(c);
        if (st == PACC_OK) st = gbgc_pump(c);
        if (st != PACC_OK) return st;
        if (v.running) {
            const cudaError_t e = cudaEventQuery(v.ev_done);
            if (e != cudaSuccess && e != cudaErrorNotReady) return cuda_ok(c, e, "gbgc serving launch") ? 0 : PACC_ECUDA;
        }
    }
    int k = 0;
    const int N = c->M.N;
    while (k < max && !v.done.empty()) {
        GbgcServer::Done& d = v.done.front();
        pacc_gbgc_result& r = out[k];
        int32_t* mz = r.max_z;
        int8_t* mb = r.max_b;
        double *pb = r.post_b, *pz = r.post_z;
        r = d.r;
        r.max_z = mz; r.max_b = mb; r.post_b = pb; r.post_z = pz; r.trace = nullptr;
        if (d.r.status == PACC_OK) {
            if (mz) std::memcpy(mz, d.max_z.data(), sizeof(int32_t) * 3 * N);
            if (mb) std::memcpy(mb, d.max_b.data(), 3 * N);
            if (pb) std::memcpy(pb, d.post_b.data(), sizeof(double) * 3 * N);
            if (pz) std::memcpy(pz, d.post_z.data(), sizeof(double) * 12 * N);
        }
        v.done.pop_front();
        k++;
    }
    return k;
}

int pacc_gbgc_run(pacc_ctx* c, const pacc_gbgc_opts* go, const pacc_element_batch* b, pacc_gbgc_result* out) {
    if (!c) return PACC_EINVAL;
    if (!go || !b || !out || b->n_elements < 0 || (b->n_elements > 0 && (!b->lengths || !b->offsets || !b->bases))) {
        c->err = "gbgc_run: options, batch and results must be non-null";
        return PACC_EINVAL;
    }
    if (go->burnin < 0 || go->mcmc < 2 || go->burnin + go->mcmc < 2 || go->prop_c <= 1 || go->prop_n <= 1 ||
        go->prop_gc <= 0) {
        c->err = "gbgc_run: burnin >= 0, mcmc >= 2, prop_c and prop_n > 1, prop_gc > 0";
        return PACC_EINVAL;
    }
    if (!c->gpu_ok) { c->err = "gbgc_run: no usable GPU"; return PACC_ECUDA; }
    const HostModel& M = c->M;
    const int S = M.S, N = M.N, n = b->n_elements;
    const int T = go->burnin + go->mcmc;
    std::vector<uint8_t> target(N, 0);
    for (int i = 0; i < go->n_target; i++)
        if (go->target && go->target[i] >= 0 && go->target[i] < N) target[go->target[i]] = 1;
    // host preprocessing, in parallel over elements
    std::vector<GbgcElem> E(n);
    std::vector<GbgcElemHdr> hdr(n);
    std::vector<std::vector<uint8_t>> blobs(n);
    {
        const int nth = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
        std::atomic<int> next(0);
        std::vector<std::thread> th;
        for (int t = 0; t < nth; t++)
            th.emplace_back([&]() {
                for (int i = next++; i < n; i = next++) {
                    gbgc_prepare(M, b->bases + b->offsets[i], b->lengths[i], (char)go->gapchar, go->missing_thres,
                                 go->conserve_prop, E[i]);
                    if (!E[i].filtered) {
                        int nint = 0;
                        for (int s : E[i].nodes) nint += s >= S;
                        if (nint == 0) E[i].filtered = 2;
                    }
                    if (!E[i].filtered) gbgc_blob(M, E[i], hdr[i], blobs[i]);
                }
            });
        for (auto& t : th) t.join();
    }
    std::vector<int> run;   // elements that reach the device
    for (int i = 0; i < n; i++) {
        pacc_gbgc_result& r = out[i];
        r.element_no = b->element_no ? b->element_no[i] : i;
        r.status = E[i].filtered ? PACC_FILTERED : PACC_OK;
        r.root = E[i].filtered ? -1 : E[i].root;
        if (!E[i].filtered) run.push_back(i);
    }
    if (run.empty()) return PACC_OK;
    // the device queue takes the longest elements first (a shorter tail)
    std::stable_sort(run.begin(), run.end(), [&](int a, int b2) { return E[a].GG > E[b2].GG; });
    if (!cuda_ok(c, cudaSetDevice(c->device), "gbgc_run: cudaSetDevice")) return PACC_ECUDA;
    const int prec = (c->o.precision == PACC_FP32 || c->o.precision == PACC_FP32_WARP) ? 1 : 0;
    int GGp_max = 32;
    for (int i : run) GGp_max = std::max(GGp_max, E[i].GGp);
    const size_t smem = gbgc_chain_smem(N, prec);
    // register budget of the chain kernel: opts.register_budget 168, else 96
    const int regs = c->o.register_budget == 168 ? 168 : 96;
    const int per_sm = gbgc_chain_occupancy(prec, regs, smem);
    if (per_sm <= 0) { c->err = "gbgc_run: the chain kernel does not fit on an SM"; return PACC_ECUDA; }
    const GbgcWs W = GbgcWs::make(N, S - 1, GGp_max, gbgc_chain_warps(), prec ? 4 : 8);
    const size_t tzb_el = (size_t)3 * T * 2 * N;
    // elements per launch: bounded by the traces' budget (opts.memory_budget_bytes, else 16 GB)
    const size_t budget = c->o.memory_budget_bytes > 0 ? (size_t)c->o.memory_budget_bytes : ((size_t)16 << 30);
    const int grid_full = c->n_sm * per_sm;
    int chunk = (int)std::max<size_t>(1, std::min<size_t>(run.size(), budget / (tzb_el + 256)));
    const int grid = std::max(1, std::min(grid_full, chunk));
    // device buffers
    size_t blob_total = 0;
    for (int i : run) blob_total += blobs[i].size();
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t o_hdr = 0, o_blob = up(sizeof(GbgcElemHdr) * run.size());
    const size_t o_tgt = up(o_blob + blob_total), o_ctr = up(o_tgt + N);
    const size_t o_ws = up(o_ctr + 256);
    const size_t o_trd = up(o_ws + W.total * (size_t)grid);
    const size_t o_tzb = up(o_trd + (size_t)chunk * 3 * 4 * T * 8);
    const size_t o_mzb = up(o_tzb + (size_t)chunk * tzb_el);
    const size_t o_mll = up(o_mzb + (size_t)chunk * 3 * 2 * N);
    const size_t o_st = up(o_mll + (size_t)chunk * 3 * 8);
    const size_t o_ph = up(o_st + (size_t)chunk * 4);
    const size_t total = up(o_ph + 9 * 8);
    char* dev = nullptr;
    if (!cuda_ok(c, cudaMalloc((void**)&dev, total), "gbgc_run: cudaMalloc")) return PACC_OOM;
    cudaStream_t st = c->stream;
    std::vector<uint8_t> hblob(blob_total);
    std::vector<GbgcElemHdr> hh(run.size());
    {
        size_t off = 0;
        for (size_t k = 0; k < run.size(); k++) {
            hh[k] = hdr[run[k]];
            hh[k].blob_off = (int64_t)off;
            std::memcpy(hblob.data() + off, blobs[run[k]].data(), blobs[run[k]].size());
            off += blobs[run[k]].size();
        }
    }
    GbgcChainParams p;
    std::memset(&p, 0, sizeof(p));
    p.T = T; p.burn = go->burnin; p.mcmc = go->mcmc; p.seed = go->seed; p.chain = go->chain;
    p.conserve_rate = go->conserve_rate; p.acce_rate = go->acce_rate; p.init_gc = go->init_gc;
    p.ca = go->conserve_prior_a; p.cb = go->conserve_prior_b;
    p.na = go->acce_prior_a; p.nb = go->acce_prior_b; p.nshift = go->acce_prior_shift;
    p.gca = go->gc_prior_a; p.gcb = go->gc_prior_b; p.gcc = go->gc_prior_c;
    p.lrate = go->prep_lrate; p.grate = go->prep_grate; p.c2m = go->cons_to_mis; p.nc2m = go->ncons_to_mis;
    p.prop_c = go->prop_c; p.prop_n = go->prop_n; p.prop_gc = go->prop_gc;
    std::memcpy(p.Q0, M.rate, sizeof(p.Q0));
    std::memcpy(p.pi, M.pi, sizeof(p.pi));
    p.target = (const uint8_t*)(dev + o_tgt);
    p.ws = dev + o_ws; p.ws_stride = W.total;
    p.N_max = N; p.n_int_max = S - 1; p.GGp_max = GGp_max;
    p.next_elem = (int*)(dev + o_ctr);
    p.tr_d = (double*)(dev + o_trd); p.tr_zb = (int8_t*)(dev + o_tzb); p.max_zb = (int8_t*)(dev + o_mzb);
    p.max_ll = (double*)(dev + o_mll); p.status = (int32_t*)(dev + o_st);
    p.phase = (unsigned long long*)(dev + o_ph);
    p.flop = p.phase + 8;
    bool ok = cuda_ok(c, cudaMemsetAsync(dev + o_ph, 0, 72, st), "memset") &&
              cuda_ok(c, cudaMemcpyAsync(dev + o_hdr, hh.data(), sizeof(GbgcElemHdr) * hh.size(), cudaMemcpyHostToDevice, st), "H2D") &&
              cuda_ok(c, cudaMemcpyAsync(dev + o_blob, hblob.data(), blob_total, cudaMemcpyHostToDevice, st), "H2D") &&
              cuda_ok(c, cudaMemcpyAsync(dev + o_tgt, target.data(), N, cudaMemcpyHostToDevice, st), "H2D");
    std::vector<double> trd((size_t)chunk * 3 * 4 * T), mll((size_t)chunk * 3);
    std::vector<int8_t> tzb((size_t)chunk * tzb_el), mzb((size_t)chunk * 3 * 2 * N);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ok = ok && cuda_ok(c, cudaEventCreate(&e0), "event") && cuda_ok(c, cudaEventCreate(&e1), "event");
    for (size_t c0 = 0; ok && c0 < run.size(); c0 += chunk) {
        const int nc = (int)std::min<size_t>(chunk, run.size() - c0);
        p.hdr = (const GbgcElemHdr*)(dev + o_hdr) + c0;
        p.blob = (const uint8_t*)(dev + o_blob);
        p.n_elem = nc;
        float ms = 0;
        ok = cuda_ok(c, cudaMemsetAsync(dev + o_ctr, 0, 256, st), "memset") &&
             cuda_ok(c, cudaEventRecord(e0, st), "event") &&
             cuda_ok(c, launch_gbgc_chain(p, std::min(grid, nc), smem, prec, regs, st), "gbgc_run: launch") &&
             cuda_ok(c, cudaEventRecord(e1, st), "event") &&
             cuda_ok(c, cudaMemcpyAsync(trd.data(), dev + o_trd, (size_t)nc * 3 * 4 * T * 8, cudaMemcpyDeviceToHost, st), "D2H") &&
             cuda_ok(c, cudaMemcpyAsync(tzb.data(), dev + o_tzb, (size_t)nc * tzb_el, cudaMemcpyDeviceToHost, st), "D2H") &&
             cuda_ok(c, cudaMemcpyAsync(mzb.data(), dev + o_mzb, (size_t)nc * 3 * 2 * N, cudaMemcpyDeviceToHost, st), "D2H") &&
             cuda_ok(c, cudaMemcpyAsync(mll.data(), dev + o_mll, (size_t)nc * 3 * 8, cudaMemcpyDeviceToHost, st), "D2H") &&
             cuda_ok(c, cudaStreamSynchronize(st), "gbgc_run") && cuda_ok(c, cudaEventElapsedTime(&ms, e0, e1), "event");
        if (!ok) break;
        c->counters.kernel_ms += ms;
        // Eval2 and Output_init per element and model, in parallel over elements
        const int nth = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
        std::atomic<int> next(0);
        std::vector<std::thread> th;
        for (int t = 0; t < nth; t++)
            th.emplace_back([&]() {
                for (int k = next++; k < nc; k = next++) {
                    const int i = run[c0 + k];
                    pacc_gbgc_result& r = out[i];
                    r.device_ms = ms / nc;
                    gbgc_finish(*go, N, E[i], trd.data() + (size_t)k * 3 * 4 * T, tzb.data() + (size_t)k * tzb_el,
                                mzb.data() + (size_t)k * 3 * 2 * N, mll.data() + (size_t)k * 3, r);
                }
            });
        for (auto& t : th) t.join();
    }
    if (ok) {   // cycles per phase of the chain kernel, summed over elements (pacc_counters.phase_cycles)
        unsigned long long ph[9];
        if (cuda_ok(c, cudaMemcpy(ph, dev + o_ph, sizeof(ph), cudaMemcpyDeviceToHost), "D2H")) {
            for (int q = 0; q < 8; q++) c->counters.phase_cycles[q] += (double)ph[q];
            c->counters.flop += (double)ph[8];
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(dev);
    return ok ? PACC_OK : PACC_ECUDA;
}

int pacc_gbgc_engine(pacc_ctx* c, const uint8_t* bases, int32_t length, int32_t gapchar, double missing_thres,
                     const int32_t* z, const int32_t* bflag, double sel_c, double sel_n, double gc_bias, double* logp,
                     double* col, double* counts, int32_t* root, uint8_t* missing, int32_t* filtered) {
    if (!c) return PACC_EINVAL;
    const int S = c->M.S, N = c->M.N;
    if (!bases || length <= 0 || !z || !bflag || !logp || !col || !counts || !root || !missing || !filtered) {
        c->err = "gbgc_engine: length must be positive and every array non-null";
        return PACC_EINVAL;
    }
    if (!c->gpu_ok) { c->err = "gbgc_engine: no usable GPU"; return PACC_ECUDA; }
    GbgcElem E;
    gbgc_prepare(c->M, bases, length, (char)gapchar, missing_thres, c->o.conserve_prop, E);
    *filtered = E.filtered;
    for (int s = 0; s < N; s++) missing[s] = (uint8_t)E.missing[s];
    if (E.filtered) return PACC_FILTERED;
    // the state of every branch of the element's tree (other nodes are not read)
    for (size_t k = 0; k + 1 < E.nodes.size(); k++) {
        const int s = E.nodes[k];
        if (z[s] < 0 || z[s] > 2 || (bflag[s] != 0 && bflag[s] != 1) || (z[s] == 2 && E.fixed[s])) {
            c->err = "gbgc_engine: z must be 0..2 (0..1 on the outgroup path) and b 0 or 1 on node " +
                     std::to_string(s);
            return PACC_EINVAL;
        }
    }
    *root = E.root;
    if (!cuda_ok(c, cudaSetDevice(c->device), "gbgc_engine: cudaSetDevice")) return PACC_ECUDA;
    const int prec = (c->o.precision == PACC_FP32 || c->o.precision == PACC_FP32_WARP) ? 1 : 0;
    const size_t rb = prec ? 4 : 8;
    const int warps = std::max(1, std::min(8, E.GGp / 32));
    const int GGp = E.GGp, nn = (int)E.nodes.size();
    // one device allocation: host-built inputs first, then outputs and scratch
    std::vector<int16_t> i16((size_t)nn + 3 * N);
    for (int k = 0; k < nn; k++) i16[k] = (int16_t)E.nodes[k];
    for (int s = 0; s < N; s++) {
        i16[nn + s] = (int16_t)E.c2a[s];
        i16[nn + N + s] = (int16_t)E.c2b[s];
        i16[nn + 2 * N + s] = (int16_t)E.par[s];
    }
    std::vector<int32_t> cls(N);
    std::vector<uint8_t> u8(2 * (size_t)N);
    for (int s = 0; s < N; s++) {
        cls[s] = 0;
        u8[s] = (uint8_t)E.missing[s];
        u8[N + s] = (uint8_t)E.fixed[s];
    }
    for (size_t k = 0; k + 1 < E.nodes.size(); k++) cls[E.nodes[k]] = z[E.nodes[k]] + 3 * bflag[E.nodes[k]];
    auto up16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
    size_t o = 0;
    const size_t o_d2 = o;     o += up16(8 * (size_t)N);
    const size_t o_logp = o;   o += up16(8 * 96 * (size_t)N);
    const size_t o_pm = o;     o += up16(rb * 96 * (size_t)N);
    const size_t o_col = o;    o += up16(8 * (size_t)GGp);
    const size_t o_cnt = o;    o += up16(8 * 16 * (size_t)N);
    const size_t o_wc = o;     o += up16(8 * 16 * (size_t)N * warps);
    const size_t o_part = o;   o += up16(rb * 4 * (size_t)N * GGp);
    const size_t o_scl = o;    o += up16(4 * (size_t)N * GGp);
    const size_t o_cls = o;    o += up16(4 * (size_t)N);
    const size_t o_i16 = o;    o += up16(2 * i16.size());
    const size_t o_u8 = o;     o += up16(u8.size());
    const size_t o_mask = o;   o += up16(E.masks.size());
    char* dev = nullptr;
    if (!cuda_ok(c, cudaMalloc((void**)&dev, o), "gbgc_engine: cudaMalloc")) return PACC_OOM;
    cudaStream_t st = c->aux;
    GbgcParams p;
    std::memset(&p, 0, sizeof(p));
    p.S = S; p.N = N; p.GG = E.GG; p.GGp = GGp; p.root = E.root; p.n_nodes = nn; p.warps = warps;
    p.nodes = (const int16_t*)(dev + o_i16);
    p.c0 = p.nodes + nn; p.c1 = p.c0 + N; p.parent = p.c1 + N;
    p.missing = (const uint8_t*)(dev + o_u8); p.fixed = p.missing + N;
    p.dist = (const double*)(dev + o_d2);
    p.cls = (const int32_t*)(dev + o_cls);
    p.masks = (const uint8_t*)(dev + o_mask);
    std::memcpy(p.Q0, c->M.rate, sizeof(p.Q0));
    std::memcpy(p.pi, c->M.pi, sizeof(p.pi));
    p.sc = sel_c; p.sn = sel_n; p.gb = gc_bias;
    p.logp = (double*)(dev + o_logp); p.pmat = dev + o_pm;
    p.col = (double*)(dev + o_col); p.counts = (double*)(dev + o_cnt); p.wcounts = (double*)(dev + o_wc);
    p.part = dev + o_part; p.scl = (int32_t*)(dev + o_scl);
    // logp and the matrices start at zero: classes that are not built stay 0,
    // as the reference's zero-initialised caches do
    bool ok = cuda_ok(c, cudaMemsetAsync(dev + o_logp, 0, o_col - o_logp, st), "gbgc_engine: memset") &&
              cuda_ok(c, cudaMemcpyAsync(dev + o_d2, E.d2.data(), 8 * (size_t)N, cudaMemcpyHostToDevice, st), "H2D") &&
              cuda_ok(c, cudaMemcpyAsync(dev + o_cls, cls.data(), 4 * (size_t)N, cudaMemcpyHostToDevice, st), "H2D") &&
              cuda_ok(c, cudaMemcpyAsync(dev + o_i16, i16.data(), 2 * i16.size(), cudaMemcpyHostToDevice, st), "H2D") &&
              cuda_ok(c, cudaMemcpyAsync(dev + o_u8, u8.data(), u8.size(), cudaMemcpyHostToDevice, st), "H2D") &&
              cuda_ok(c, cudaMemcpyAsync(dev + o_mask, E.masks.data(), E.masks.size(), cudaMemcpyHostToDevice, st), "H2D") &&
              cuda_ok(c, launch_gbgc(p, prec, st), "gbgc_engine: launch") &&
              cuda_ok(c, cudaMemcpyAsync(logp, dev + o_logp, 8 * 96 * (size_t)N, cudaMemcpyDeviceToHost, st), "D2H") &&
              cuda_ok(c, cudaMemcpyAsync(col, dev + o_col, 8 * (size_t)E.GG, cudaMemcpyDeviceToHost, st), "D2H") &&
              cuda_ok(c, cudaMemcpyAsync(counts, dev + o_cnt, 8 * 16 * (size_t)N, cudaMemcpyDeviceToHost, st), "D2H") &&
              cuda_ok(c, cudaStreamSynchronize(st), "gbgc_engine");
    cudaFree(dev);
    return ok ? PACC_OK : PACC_ECUDA;
}

int pacc_debug_pmatrix(pacc_ctx* c, int n, const double* d, const double* r, double* out) {
    if (!c || n <= 0) return PACC_EINVAL;
    if (!c->gpu_ok) return PACC_ECUDA;
    cudaSetDevice(c->device);
    if (!ensure_model(c)) return PACC_ECUDA;
    double *dd = nullptr, *dr = nullptr, *dout = nullptr;
    if (!cuda_ok(c, cudaMalloc(&dd, n * 8), "malloc") || !cuda_ok(c, cudaMalloc(&dr, n * 8), "malloc") ||
        !cuda_ok(c, cudaMalloc(&dout, (size_t)n * 128), "malloc")) {
        cudaFree(dd); cudaFree(dr); cudaFree(dout);     // cudaFree(nullptr) is a no-op
        return PACC_OOM;
    }
    // inputs on the kernel's stream: a plain cudaMemcpy from pageable memory
    // may still be in flight when a kernel on a non-blocking stream starts
    cudaMemcpyAsync(dd, d, n * 8, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dr, r, n * 8, cudaMemcpyHostToDevice, c->stream);
    cudaError_t e = launch_pmatrix(n, dd, dr, dout, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, (size_t)n * 128, cudaMemcpyDeviceToHost);
    cudaFree(dd); cudaFree(dr); cudaFree(dout);
    return cuda_ok(c, e, "pmatrix") ? PACC_OK : PACC_ECUDA;
}

int pacc_pmatrix_noalloc(pacc_ctx* c, int n, const double* d, const double* r, double* out) {
    if (!c) return PACC_EINVAL;
    if (n <= 0 || n > PACC_NOALLOC_MAX_PAIRS || !d || !r || !out) {
        c->err = "pmatrix_noalloc: n must be in 1.." + std::to_string(PACC_NOALLOC_MAX_PAIRS) +
                 " and d, r, out non-null";
        return PACC_EINVAL;
    }
    if (!c->gpu_ok) { c->err = "pmatrix_noalloc: no usable GPU"; return PACC_ECUDA; }
    if (!cuda_ok(c, cudaSetDevice(c->device), "pmatrix_noalloc: cudaSetDevice")) return PACC_ECUDA;
    // returns at once when this context's model is the device's (it may be
    // serving); otherwise the other context's launch is waited for
    if (!ensure_model(c)) return PACC_ECUDA;
    // the scratch's device address, looked up on every call (a lookup after
    // the module is loaded is cheap, and it stays right across a device reset)
    double* base = nullptr;
    if (!cuda_ok(c, noalloc_scratch_address(&base), "pmatrix_noalloc: cudaGetSymbolAddress")) return PACC_ECUDA;
    const size_t M = PACC_NOALLOC_MAX_PAIRS;
    double* sd = base;
    double* sr = base + M;
    double* so = base + 2 * M;
    // the context's own second stream: a serving launch on the main stream
    // does not hold this call back
    cudaStream_t st = c->aux;
    cudaError_t e = cudaMemcpyAsync(sd, d, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sr, r, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_pmatrix(n, sd, sr, so, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, so, sizeof(double) * 16 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cuda_ok(c, e, "pmatrix_noalloc") ? PACC_OK : PACC_ECUDA;
}

int pacc_debug_encode(pacc_ctx* c, const uint8_t* bases, int32_t length, int8_t* tg_out, int32_t* n_cols,
                      uint8_t* missing_out, int32_t* root_out, int32_t* filtered) {
    if (!c) return PACC_EINVAL;
    HostElem E;
    if (!preprocess(c->M, c->o, bases, length, E, true)) return PACC_EINVAL;
    *filtered = E.filtered ? 1 : 0;
    if (E.filtered) { *n_cols = 0; return PACC_OK; }
    *n_cols = E.GG;
    std::memcpy(tg_out, E.tg_full.data(), E.tg_full.size());
    for (int s = 0; s < c->M.N; s++) missing_out[s] = E.missing[s];
    *root_out = E.root;
    return PACC_OK;
}

int pacc_debug_patterns(pacc_ctx* c, const uint8_t* bases, int32_t length, int32_t* pattern_of, int32_t* weights,
                        int32_t* n_cols, int32_t* n_patterns) {
    if (!c || !bases || !pattern_of || !weights || !n_cols || !n_patterns) return PACC_EINVAL;
    HostElem E;
    if (!preprocess(c->M, c->o, bases, length, E, false)) return PACC_EINVAL;
    if (E.filtered) { *n_cols = 0; *n_patterns = 0; return PACC_FILTERED; }
    *n_cols = E.GG;
    *n_patterns = E.GGu;
    std::memcpy(pattern_of, E.pattern_of.data(), sizeof(int32_t) * E.GG);
    std::memcpy(weights, E.pw.data(), sizeof(int32_t) * E.GGu);
    return PACC_OK;
}

int pacc_debug_loglik(pacc_ctx* c, const uint8_t* bases, int32_t length, const int32_t* z, double c_rate,
                      double n_rate, double* out, int32_t* n_cols) {
    if (!c) return PACC_EINVAL;
    if (!c->gpu_ok) return PACC_ECUDA;
    cudaSetDevice(c->device);
    if (!ensure_model(c)) return PACC_ECUDA;
    HostElem E;
    if (!preprocess(c->M, c->o, bases, length, E, false)) return PACC_EINVAL;
    if (E.filtered) { *n_cols = 0; return PACC_FILTERED; }
    const int N = c->M.N;
    const int prec = (c->o.precision == PACC_FP32 || c->o.precision == PACC_FP32_WARP) ? 1 : 0;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    ElemHeader H;
    std::memset(&H, 0, sizeof(H));
    H.GG = E.GG; H.GGp = E.GGp; H.root = E.root; H.n_nodes = E.n_nodes; H.n_int = E.n_int;
    size_t off = 0;
    H.codes_off = off; off = al(off + E.codes.size());
    H.tg_off = off; off = al(off + E.tg0.size());
    H.prefix_off = off; off = al(off + E.prefix.size() * 4);
    H.topo_off = off; off = al(off + topo_bytes(N));
    std::vector<uint8_t> blob(off);
    std::memcpy(&blob[H.codes_off], E.codes.data(), E.codes.size());
    std::memcpy(&blob[H.tg_off], E.tg0.data(), E.tg0.size());
    std::memcpy(&blob[H.prefix_off], E.prefix.data(), E.prefix.size() * 4);
    std::memcpy(&blob[H.topo_off], E.topo.data(), E.topo.size() * 2);
    std::memcpy(&blob[H.topo_off + ((E.topo.size() * 2 + 15) & ~(size_t)15)], E.dist2.data(), N * 8);
    size_t ws = ws_bytes(E.n_int, E.GGp, 1, 1, N, prec);
    void *dblob = nullptr, *dh = nullptr, *dws = nullptr, *dz = nullptr, *dout = nullptr;
    cudaError_t e = cudaMalloc(&dblob, off);
    if (e == cudaSuccess) e = cudaMalloc(&dh, sizeof(H));
    if (e == cudaSuccess) e = cudaMalloc(&dws, ws);
    if (e == cudaSuccess) e = cudaMalloc(&dz, N * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dout, (size_t)E.GG * 8);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dblob, blob.data(), off, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dh, &H, sizeof(H), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dz, z, N * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        ChainParams p;
        std::memset(&p, 0, sizeof(p));
        p.hdr = (const ElemHeader*)dh;
        p.blob = (const uint8_t*)dblob;
        p.n_elem = 1;
        p.ws = (char*)dws;
        p.ws_stride = ws;
        p.n_int_max = E.n_int;
        p.GGp_max = E.GGp;
        p.stack_cap = c->stack_cap;
        int BT = 128;
        e = launch_loglik(p, (const int32_t*)dz, c_rate, n_rate, (double*)dout, BT, smem_bytes(N, BT, prec, c->stack_cap), prec,
                          c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e == cudaSuccess) e = cudaMemcpy(out, dout, (size_t)E.GG * 8, cudaMemcpyDeviceToHost);
    }
    cudaFree(dblob); cudaFree(dh); cudaFree(dws); cudaFree(dz); cudaFree(dout);
    *n_cols = E.GG;
    return cuda_ok(c, e, "loglik") ? PACC_OK : PACC_ECUDA;
}

int pacc_debug_stream(uint32_t seed, uint64_t w0, int n, uint32_t* out) {
    if (n <= 0) return PACC_EINVAL;
    uint32_t* d = nullptr;
    if (cudaMalloc(&d, (size_t)n * 4) != cudaSuccess) return PACC_OOM;
    cudaError_t e = launch_stream(seed, w0, n, d, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(out, d, (size_t)n * 4, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? PACC_OK : PACC_ECUDA;
}

int pacc_measure_fma_peak(int device, double* fp64, double* fp32) {
    if (cudaSetDevice(device) != cudaSuccess) return PACC_ECUDA;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    void* d = nullptr;
    if (cudaMalloc(&d, 1 << 20) != cudaSuccess) return PACC_OOM;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    double res[2] = {0, 0};
    for (int prec = 0; prec < 2; prec++) {
        int grid = nsm * 8, BT = 256;
        int iters = prec == 0 ? 2000 : 40000;
        launch_fma_probe(prec, grid, BT, iters / 10, d, 0);
        cudaDeviceSynchronize();
        float best = 1e30f;
        for (int rep = 0; rep < 3; rep++) {
            cudaEventRecord(a);
            launch_fma_probe(prec, grid, BT, iters, d, 0);
            cudaEventRecord(b);
            cudaEventSynchronize(b);
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            best = std::min(best, ms);
        }
        res[prec] = (double)grid * BT * iters * 8.0 * 2.0 / (best * 1e-3);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(d);
    if (fp64) *fp64 = res[0];
    if (fp32) *fp32 = res[1];
    return cudaGetLastError() == cudaSuccess ? PACC_OK : PACC_ECUDA;
}

}  // extern "C"
