"""Load a golden case (tests/golden/<case>/) into a synth.Dataset + PaccOpts,
and read the reference's output tables and traces stored with it."""
from __future__ import annotations

import os

import numpy as np

from phyloacc_gb300 import abi, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["st12_default", "st12_options", "st43_default", "st12_priors", "st12_filters"]


def _parse_newick(s, i, nodes):
    kids = []
    if s[i] == "(":
        i += 1
        while True:
            k, i = _parse_newick(s, i, nodes)
            kids.append(k)
            if s[i] == ",":
                i += 1
                continue
            if s[i] == ")":
                i += 1
                break
    a = i
    while i < len(s) and s[i] not in ":,);":
        i += 1
    name = s[a:i]
    dist = 0.0
    if i < len(s) and s[i] == ":":
        i += 1
        b = i
        while i < len(s) and s[i] not in ",);":
            i += 1
        dist = float(np.float32(float(s[b:i])))
    nodes.append({"name": name, "dist": dist, "kids": kids})
    return len(nodes) - 1, i


def read_mod(path):
    pi = Q = newick = None
    lines = open(path).read().split("\n")
    k = 0
    while k < len(lines):
        ln = lines[k].strip()
        if ln.startswith("BACKGROUND:"):
            pi = np.array([float(x) for x in ln.split()[1:5]])
        elif ln.startswith("RATE_MAT:"):
            Q = np.array([[float(x) for x in lines[k + 1 + r].split()] for r in range(4)])
            k += 4
        elif ln.startswith("TREE:"):
            newick = ln.split()[1]
        k += 1
    nodes = []
    _parse_newick(newick, 0, nodes)
    S = sum(1 for n in nodes if not n["kids"])
    N = 2 * S - 1
    leaf, br = 0, S
    for n in nodes:
        if n["kids"]:
            n["id"] = br
            br += 1
        else:
            n["id"] = leaf
            leaf += 1
    children = np.full((N, 2), -1, np.int32)
    dist = np.zeros(N)
    names = [""] * N
    for n in nodes:
        names[n["id"]] = n["name"]
        dist[n["id"]] = n["dist"]
        if n["kids"]:
            children[n["id"]] = sorted(nodes[k]["id"] for k in n["kids"])
    return synth.Tree(S, children, dist, names, newick), pi, Q


def read_cfg(path):
    kv = {}
    for ln in open(path):
        w = ln.split()
        if len(w) == 2 and not w[0].startswith("#"):
            kv[w[0]] = w[1]
    return kv


def opts_from_cfg(kv):
    o = abi.default_opts()
    f = {"BURNIN": ("burnin", int), "MCMC": ("mcmc", int), "SEED": ("seed", int), "ADAPT_FREQ": ("adapt_freq", int),
         "INIT_CONSERVE_RATE": ("init_conserve_rate", float), "INIT_ACCE_RATE": ("init_acce_rate", float),
         "CONSERVE_PRIOR_A": ("conserve_prior_a", float), "CONSERVE_PRIOR_B": ("conserve_prior_b", float),
         "ACCE_PRIOR_A": ("acce_prior_a", float), "ACCE_PRIOR_B": ("acce_prior_b", float),
         "ROPT": ("ropt", int), "CUB": ("cub", float), "NLB": ("nlb", float),
         "INIT_LRATE": ("init_lrate", float), "INIT_LRATE2": ("init_lrate2", float), "INIT_GRATE": ("init_grate", float),
         "HYPER_LRATE_A": ("hyper_lrate_a", float), "HYPER_LRATE_B": ("hyper_lrate_b", float),
         "HYPER_GRATE_A": ("hyper_grate_a", float), "HYPER_GRATE_B": ("hyper_grate_b", float),
         "HYPER_LRATE2_A": ("hyper_lrate2_a", float), "HYPER_LRATE2_B": ("hyper_lrate2_b", float),
         "CONSERVE_PROP": ("conserve_prop", float), "GAP_PROP": ("gap_prop", float),
         "CONSTOMIS": ("cons_to_mis", float), "TRIM_GAP_PERCENT": ("trim_gap_percent", float),
         "MIN_LEN": ("min_len", int)}
    for k, v in kv.items():
        if k in f:
            setattr(o, f[k][0], f[k][1](v))
        elif k == "PRUNE_TREE":
            o.prune_tree = 1 if v in ("1", "true") else 0
        elif k == "GAPCHAR":
            o.gapchar = ord(v[0])
    if o.hyper_lrate2_a == 0:
        o.init_lrate2 = 0.0
    return o


def load_case(name):
    d = os.path.join(GOLDEN, name)
    kv = read_cfg(os.path.join(d, "case.cfg"))
    tree, pi, Q = read_mod(os.path.join(d, kv["PHYTREE_FILE"]))
    S = tree.n_species
    seqs = {}
    cur = None
    for ln in open(os.path.join(d, kv["ALIGN_FILE"])):
        ln = ln.strip()
        if ln.startswith(">"):
            cur = ln[1:].strip()
            seqs[cur] = []
        elif cur is not None:
            seqs[cur].append(ln.lower())
    rows = [np.frombuffer("".join(seqs[tree.names[s]]).encode(), np.uint8) for s in range(S)]
    names, lens = [], []
    for ln in open(os.path.join(d, kv["SEG_FILE"])):
        w = ln.strip().split("\t")
        if len(w) < 3:
            break
        names.append(w[0])
        lens.append(int(w[2]) - int(w[1]))
    lens = np.array(lens, np.int32)
    E = len(lens)
    offsets = np.zeros(E, np.int64)
    offsets[1:] = np.cumsum(lens[:-1].astype(np.int64) * S)
    bases = np.empty(int(lens.sum()) * S, np.uint8)
    start = 0
    for e in range(E):
        blk = np.stack([r[start:start + lens[e]] for r in rows])
        bases[offsets[e]:offsets[e] + blk.size] = blk.reshape(-1)
        start += lens[e]

    def ids(key):
        out = []
        for t in kv.get(key, "").split(";"):
            if t:
                out.append(tree.names.index(t) if t in tree.names[:S] else S)
        return out

    ds = synth.Dataset(tree, pi, Q, ids("OUTGROUP"), ids("CONSERVE"), ids("TARGETSPECIES"), lens, offsets, bases,
                       names, np.zeros(E, bool), np.zeros(E), np.zeros(E))
    return ds, opts_from_cfg(kv), kv


def read_table(path):
    lines = [ln.rstrip("\n").split("\t") for ln in open(path)]
    return lines[0], lines[1:]


def ref_tables(name):
    d = os.path.join(GOLDEN, name, "out")
    out = {}
    for f in sorted(os.listdir(d)):
        out[f[len("case_"):-4]] = read_table(os.path.join(d, f))
    return out


def ref_traces(name):
    z = np.load(os.path.join(GOLDEN, name, "traces.npz"))
    return {k: z[k] for k in z.files}


def as_float(x):
    return float(x.replace("-nan", "nan"))
