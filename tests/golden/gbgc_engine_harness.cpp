// Harness over the unmodified PhyloAcc-ST-GBGC sources (the gBGC model):
// builds the reference's model object (BPP) and per-element object (BPP_C)
// from a .mod / FASTA / bed triple as its main.cpp does, sets chosen latent
// states and rates, and writes what the reference's own functions compute
// from them:
//   * the six per-branch log transition matrices of init_cache_TM
//     (bpp_c.cpp:1563-1621) for Q(s, b) of getRate (bpp_c.cpp:13-30);
//   * the per-column log-likelihood after the pruning pass of Update_Tg
//     (bpp_c.cpp:477-540, tosample = false);
//   * the expected (child base, parent base) counts of the sampling pass of
//     Update_Tg (bpp_c.cpp:541-596, tosample = true), posterior_Tg_next.
// The private members it sets are reached by compiling this file (only) with
// `private` defined as `public`; the reference sources are compiled as they
// are.  Test infrastructure: the golden vectors it writes pin the oracle's
// gBGC restatement and the GPU kernels.
// standard and library headers first, so that only the reference's own
// classes are affected by the access redefinition below
#include <algorithm>
#include <armadillo>
#include <cassert>
#include <cmath>
#include <fstream>
#include <iostream>
#include <map>
#include <queue>
#include <set>
#include <sstream>
#include <stack>
#include <string>
#include <sys/time.h>
#include <vector>
#include <gsl/gsl_randist.h>
#include <gsl/gsl_rng.h>
#include <gsl/gsl_sf_gamma.h>
#define private public
#include "bpp.hpp"
#include "bpp_c.hpp"
#include "newick.h"
#include "profile.h"
#undef private

#include <cstdio>
#include <random>

int main(int argc, char** argv) {
    if (argc < 8) {
        fprintf(stderr, "usage: harness mod fa bed target outgroup conserve out [states per element]\n");
        return 1;
    }
    const int n_states = argc > 8 ? atoi(argv[8]) : 3;
    PhyloProf profile = LoadPhyloProfiles(argv[2], argv[3]);
    PhyloTree tree = LoadPhyloTree(argv[1]);
    // main.cpp:36-80 defaults of the gBGC program
    BPP bpp(0, profile, tree, ".", argv[4], argv[5], 0.8, argv[6], "", -2, 0, 0, 1, 0.6, 5, 0.4, 5, 0.4, 4, 0.8, 0.2,
            1, 1, 7728, 0.1, 0.8, 0.01, 0.1, 0.8, false);
    bpp.InitMCMC(20, 60, 100);
    FILE* out = fopen(argv[7], "w");
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    const int N = bpp.N, S = bpp.S;
    fprintf(out, "N %d S %d\n", N, S);
    for (int c = 0; c < bpp.C; c++) {
        bool filter = false;
        BPP_C e(c, profile, bpp, '*', 0.8, filter, false);
        if (filter) {
            fprintf(out, "element %d filtered\n", c);
            continue;
        }
        e.initMCMC(0, bpp, 1);
        for (int k = 0; k < n_states; k++) {
            // states: Z in {0, 1, 2} (not 2 on the outgroup path, where the
            // reference keeps no accelerated matrices), B in {0, 1}
            for (int s = 0; s < N; s++) {
                e.Z[s] = -1;
                e.isGB[s] = false;
            }
            for (int s : e.nodes) {
                const bool fixed = e.fixZ[s] == 1;
                e.Z[s] = (int)(U(rng) * (fixed ? 2 : 3));
                e.isGB[s] = U(rng) < 0.35;
            }
            const double sc = -0.5 - 2.5 * U(rng), sn = -1.0 + 3.0 * U(rng), gb = 0.1 + 2.9 * U(rng);
            std::vector<arma::mat> Qs(6);
            Qs[0] = bpp.submat;
            Qs[1] = e.getRate(bpp.submat, sc, 0);
            Qs[2] = e.getRate(bpp.submat, sn, 0);
            Qs[3] = e.getRate(bpp.submat, 0, gb);
            Qs[4] = e.getRate(bpp.submat, sc, gb);
            Qs[5] = e.getRate(bpp.submat, sn, gb);
            e.init_cache_TM(Qs);
            for (int s = S; s < N; s++)
                for (int g = 0; g < e.GG; g++) e.lambda[g][s].fill(0);
            std::vector<bool> visited(N, false);
            std::vector<double> col(e.GG);
            for (int g = 0; g < e.GG; g++) {
                e.Update_Tg(g, visited, bpp, false);
                col[g] = BPP::log_exp_sum(e.lambda[g][e.root]);
            }
            for (int s = 0; s < N; s++) e.posterior_Tg_next[s].fill(0);
            for (int g = 0; g < e.GG; g++) e.Update_Tg(g, visited, bpp, true);
            fprintf(out, "element %d state %d GG %d root %d sc %.17g sn %.17g gb %.17g\n", c, k, e.GG, e.root, sc, sn,
                    gb);
            fprintf(out, "missing");
            for (int s = 0; s < N; s++) fprintf(out, " %d", (int)e.missing[s]);
            fprintf(out, "\nnodes %zu", e.nodes.size());
            for (int s : e.nodes) fprintf(out, " %d", s);
            fprintf(out, "\nparent");
            for (int s = 0; s < N; s++) fprintf(out, " %d", e.parent2[s]);
            fprintf(out, "\nchildren");
            for (int s = 0; s < N; s++) fprintf(out, " %d %d", e.children2[s][0], e.children2[s][1]);
            fprintf(out, "\ndist");
            for (int s = 0; s < N; s++) fprintf(out, " %.17g", e.distances2[s]);
            fprintf(out, "\nZ");
            for (int s = 0; s < N; s++) fprintf(out, " %d", e.Z[s]);
            fprintf(out, "\nB");
            for (int s = 0; s < N; s++) fprintf(out, " %d", (int)e.isGB[s]);
            const std::vector<arma::mat>* caches[6] = {&e.log_cache_TM_null, &e.log_cache_TM_cons, &e.log_cache_TM_neut,
                                                       &e.log_cache_TM_null_B, &e.log_cache_TM_cons_B,
                                                       &e.log_cache_TM_neut_B};
            for (int k6 = 0; k6 < 6; k6++) {
                fprintf(out, "\nlogP%d", k6);
                for (int s = 0; s < N; s++)
                    for (int i = 0; i < 4; i++)
                        for (int j = 0; j < 4; j++) fprintf(out, " %.17g", (*caches[k6])[s](i, j));
            }
            fprintf(out, "\ncol");
            for (int g = 0; g < e.GG; g++) fprintf(out, " %.17g", col[g]);
            fprintf(out, "\ncounts");
            for (int s = 0; s < N; s++)
                for (int i = 0; i < 4; i++)
                    for (int j = 0; j < 4; j++) fprintf(out, " %.17g", e.posterior_Tg_next[s](i, j));
            fprintf(out, "\n");
        }
    }
    fclose(out);
    return 0;
}
