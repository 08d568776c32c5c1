// cli_io.h — the input side shared by the command-line drop-ins
// (phyloacc-st-gpu, phyloacc-gbgc-gpu): the .mod reader (newick.cpp of both
// programs), the FASTA + bed profile reader (profile.cpp) and small string
// helpers.  Header-only; each executable includes it once.
#pragma once
#include <dirent.h>

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

using std::string;
using std::vector;

static string trim(string s, const string& ts = " \t\n") {
    s.erase(0, s.find_first_not_of(ts));
    s.erase(s.find_last_not_of(ts) + 1);
    return s;
}

static vector<string> split(const string& s, char delim) {
    vector<string> out;
    std::stringstream ss(s);
    string item;
    while (std::getline(ss, item, delim)) out.push_back(item);
    return out;
}

static string lower(string s) {
    for (auto& ch : s) ch = (char)std::tolower((unsigned char)ch);
    return s;
}

[[noreturn]] static void die(const string& msg) {
    std::cerr << msg << std::endl;
    std::exit(1);
}

// ---------------------------------------------------------------------------
// .mod file: BACKGROUND, RATE_MAT and a labelled Newick TREE (newick.cpp:431-517)
// ---------------------------------------------------------------------------
struct TNode {
    string name;
    double dist = 0;
    vector<int> kids;
    int id = -1;
};

struct Tree {
    vector<TNode> nodes;  // parse order
    int root = -1;
    int S = 0;
    vector<string> names;       // by PhyloAcc id
    vector<double> distances;   // by id
    vector<int> children;       // [2N]
};

// Recursive Newick parser.  Branch lengths are parsed as float like the
// reference (newick.cpp:185,300,325); every node must carry a label
// (newick.cpp:416-419).
static int parse_newick(const string& s, size_t& i, Tree& T) {
    TNode nd;
    if (i < s.size() && s[i] == '(') {
        i++;
        for (;;) {
            int k = parse_newick(s, i, T);
            nd.kids.push_back(k);
            if (i < s.size() && s[i] == ',') { i++; continue; }
            if (i < s.size() && s[i] == ')') { i++; break; }
            die("(Error. Malformed tree)");
        }
    }
    size_t a = i;
    while (i < s.size() && s[i] != ':' && s[i] != ',' && s[i] != ')' && s[i] != ';') i++;
    nd.name = s.substr(a, i - a);
    if (i < s.size() && s[i] == ':') {
        i++;
        size_t b = i;
        while (i < s.size() && s[i] != ',' && s[i] != ')' && s[i] != ';') i++;
        nd.dist = (double)(float)std::atof(s.substr(b, i - b).c_str());
    }
    T.nodes.push_back(nd);
    return (int)T.nodes.size() - 1;
}

static void load_mod(const string& path, Tree& T, double pi[4], double Q[16]) {
    std::ifstream in(path.c_str());
    if (!in) die("(Error. Cannot open the phylogenetic tree input file: " + path + ")");
    string line, newick;
    for (int i = 0; i < 4; i++) pi[i] = 0;
    for (int i = 0; i < 16; i++) Q[i] = 0;
    while (std::getline(in, line)) {
        if (line == "") break;
        line = trim(line);
        vector<string> sp = split(line, ' ');
        if (sp.empty()) continue;
        if (sp[0] == "BACKGROUND:") {
            int k = 0;
            for (size_t g = 1; g < sp.size() && k < 4; g++)
                if (sp[g] != "") pi[k++] = std::atof(sp[g].c_str());
        } else if (sp[0] == "RATE_MAT:") {
            for (int r = 0; r < 4; r++) {
                if (!std::getline(in, line)) die("(Error. Truncated RATE_MAT)");
                vector<string> tk = split(trim(line), ' ');
                int k = 0;
                for (auto& t : tk)
                    if (t != "" && k < 4) Q[r * 4 + k++] = std::atof(t.c_str());
            }
        } else if (sp[0] == "TREE:" && sp.size() > 1) {
            newick = trim(sp[1]);
        }
    }
    if (newick.empty()) die("(Error. No TREE in " + path + ")");
    size_t i = 0;
    T.root = parse_newick(newick, i, T);
    // PhyloAcc ids: leaves 0..S-1, internal S..N-1, both in postorder (newick.cpp:382-400)
    int S = 0;
    for (auto& nd : T.nodes) if (nd.kids.empty()) S++;
    T.S = S;
    int N = 2 * S - 1;
    if ((int)T.nodes.size() != N) die("(Error. The tree must be binary)");
    int leaf = 0, br = S;
    // T.nodes is already in postorder (children pushed before parents)
    for (auto& nd : T.nodes) nd.id = nd.kids.empty() ? leaf++ : br++;
    T.names.assign(N, "");
    T.distances.assign(N, 0);
    T.children.assign(2 * N, -1);
    for (auto& nd : T.nodes) {
        if (nd.name.empty()) die("\n(Error. Some nodes in the tree aren't labeled. Please label all nodes and try again!)");
        T.names[nd.id] = nd.name;
        T.distances[nd.id] = nd.dist;
        vector<int> ids;
        for (int k : nd.kids) ids.push_back(T.nodes[k].id);
        std::sort(ids.begin(), ids.end());  // dag order (bpp.cpp:105-117)
        for (size_t k = 0; k < ids.size() && k < 2; k++) T.children[2 * nd.id + k] = ids[k];
    }
}

// ---------------------------------------------------------------------------
// FASTA + bed (profile.cpp:17-126)
// ---------------------------------------------------------------------------
struct Profile {
    vector<string> names, X, elem_names;
    vector<std::pair<long, long>> pos;
};

static Profile load_profile(const string& fa, const string& bed) {
    Profile P;
    std::ifstream in(fa.c_str());
    if (!in) die("(Error. Cannot open the phylogenetic profile input file: " + fa + ")");
    string line, whole;
    bool have = false;
    size_t G = 0;
    while (std::getline(in, line)) {
        line = trim(line);
        if (!line.empty() && line[0] == '>') {
            if (have) {
                if (P.X.empty()) G = whole.size();
                else if (whole.size() != G) die("(Error. Sequences of unequal length in " + fa + ")");
                P.X.push_back(lower(whole));
            }
            P.names.push_back(trim(line.substr(1)));
            whole.clear();
            have = true;
        } else {
            whole += line;
        }
    }
    if (have) {
        if (!P.X.empty() && whole.size() != G) die("(Error. Sequences of unequal length in " + fa + ")");
        P.X.push_back(lower(whole));
    }
    std::ifstream bs(bed.c_str());
    if (!bs) die("(Error. Cannot open the segment input file: " + bed + ")");
    while (std::getline(bs, line)) {
        line = trim(line);
        vector<string> sp = split(line, '\t');
        if (sp.size() < 3) break;
        P.elem_names.push_back(sp[0]);
        P.pos.push_back({std::atoi(sp[1].c_str()), std::atoi(sp[2].c_str())});
    }
    return P;
}

static bool dir_exists(const string& p) {
    if (p.empty()) return false;
    DIR* d = opendir(p.c_str());
    if (!d) return false;
    closedir(d);
    return true;
}

static vector<int> species_ids(const string& list, const vector<string>& names) {
    vector<int> out;
    for (auto& t : split(trim(list), ';')) {
        int pos = (int)(std::find(names.begin(), names.end(), t) - names.begin());
        out.push_back(pos);  // a name that is not found maps to S (bpp.hpp:230-235)
    }
    return out;
}

