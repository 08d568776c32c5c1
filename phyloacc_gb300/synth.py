"""Seeded synthetic PhyloAcc-ST inputs.

The reference measures nothing public (its own test data is fetched over the
network by bioconda_test.sh and is not shipped), so every workload here is
synthetic: a Yule tree with labelled internal nodes, a reversible (REV) rate
matrix normalised to one substitution per unit time, elements simulated down
the tree with per-branch rate multipliers (conserved r1 everywhere, accelerated
r2 on target clades), and masking by gaps / N.

Node numbering follows PhyloAcc's Newick reader: leaves 0..S-1 and internal
nodes S..N-1 in postorder of the Newick string, root N-1
(src/PhyloAcc-ST/newick.cpp:382-400); children are listed in increasing id
order (src/PhyloAcc-ST/bpp.cpp:105-117).  Branch lengths are rounded to
float32 because the reader parses them with (float)atof
(src/PhyloAcc-ST/newick.cpp:185,300,325).
"""
from __future__ import annotations

import dataclasses
import os
from typing import List, Optional

import numpy as np

BASES = np.frombuffer(b"acgt", dtype=np.uint8)


@dataclasses.dataclass
class Tree:
    n_species: int
    children: np.ndarray      # [N, 2] int32, -1 for leaves
    distances: np.ndarray     # [N] float64 (float32-representable)
    names: List[str]          # [N]
    newick: str

    @property
    def n_nodes(self) -> int:
        return 2 * self.n_species - 1

    def parent(self) -> np.ndarray:
        par = np.full(self.n_nodes, -1, dtype=np.int64)
        for i in range(self.n_nodes):
            for c in self.children[i]:
                if c >= 0:
                    par[c] = i
        return par

    def leaves_under(self, node: int) -> List[int]:
        if self.children[node, 0] < 0:
            return [node]
        out: List[int] = []
        for c in self.children[node]:
            out += self.leaves_under(int(c))
        return out

    def nodes_under(self, node: int) -> List[int]:
        if self.children[node, 0] < 0:
            return [node]
        out: List[int] = [node]
        for c in self.children[node]:
            out += self.nodes_under(int(c))
        return out


@dataclasses.dataclass
class Dataset:
    tree: Tree
    pi: np.ndarray            # [4]
    Q: np.ndarray             # [4, 4]
    outgroup: List[int]
    conserve: List[int]
    target: List[int]
    lengths: np.ndarray       # [E] int32
    offsets: np.ndarray       # [E] int64 byte offset of each element block
    bases: np.ndarray         # uint8, per element S rows x GG bytes (lower case)
    element_names: List[str]
    accelerated: np.ndarray   # [E] bool (truth)
    r1: np.ndarray            # [E] truth conserved rate
    r2: np.ndarray            # [E] truth accelerated rate (0 if none)

    @property
    def n_elements(self) -> int:
        return len(self.lengths)

    def element(self, e: int) -> np.ndarray:
        S = self.tree.n_species
        L = int(self.lengths[e])
        o = int(self.offsets[e])
        return self.bases[o:o + S * L].reshape(S, L)

    def subset(self, idx) -> "Dataset":
        idx = np.asarray(idx)
        S = self.tree.n_species
        blocks = [self.bases[int(self.offsets[i]):int(self.offsets[i]) + S * int(self.lengths[i])] for i in idx]
        lens = self.lengths[idx].astype(np.int32)
        offs = np.zeros(len(idx), dtype=np.int64)
        if len(idx) > 1:
            offs[1:] = np.cumsum(lens[:-1].astype(np.int64) * S)
        return dataclasses.replace(
            self, lengths=lens, offsets=offs,
            bases=np.concatenate(blocks) if blocks else np.zeros(0, np.uint8),
            element_names=[self.element_names[i] for i in idx],
            accelerated=self.accelerated[idx], r1=self.r1[idx], r2=self.r2[idx])


# ---------------------------------------------------------------------------
# trees
# ---------------------------------------------------------------------------
class _Node:
    __slots__ = ("kids", "length", "name", "id")

    def __init__(self):
        self.kids: List["_Node"] = []
        self.length = 0.0
        self.name = ""
        self.id = -1


def _yule(rng: np.random.Generator, n_leaves: int) -> _Node:
    root = _Node()
    active = [root]
    while len(active) < n_leaves:
        dt = rng.exponential(1.0 / len(active))
        for nd in active:
            nd.length += dt
        i = int(rng.integers(len(active)))
        nd = active.pop(i)
        a, b = _Node(), _Node()
        nd.kids = [a, b]
        active += [a, b]
    dt = rng.exponential(1.0 / len(active))
    for nd in active:
        nd.length += dt
    return root


def _height(nd: _Node) -> float:
    if not nd.kids:
        return 0.0
    return max(k.length + _height(k) for k in nd.kids)


def _number(root: _Node, S: int):
    leaf = [0]
    internal = [S]
    order: List[_Node] = []

    def rec(nd: _Node):
        for k in nd.kids:
            rec(k)
        if not nd.kids:
            nd.id = leaf[0]
            leaf[0] += 1
        else:
            nd.id = internal[0]
            internal[0] += 1
        order.append(nd)

    rec(root)
    return order


def _newick(nd: _Node, is_root=True) -> str:
    if nd.kids:
        s = "(" + ",".join(_newick(k, False) for k in nd.kids) + ")" + nd.name
    else:
        s = nd.name
    s += ":" + repr(float(np.float32(nd.length)))
    return s + (";" if is_root else "")


def make_tree(n_species: int, total_length: float, seed: int, outgroup: bool = True) -> Tree:
    """Rooted binary Yule tree; with outgroup=True the root joins one outgroup
    leaf to a Yule ingroup of n_species-1 taxa.  Branch lengths are scaled so
    that they sum to total_length."""
    rng = np.random.default_rng(seed)
    if outgroup:
        ingroup = _yule(rng, n_species - 1)
        out = _Node()
        ingroup.length = 0.25 * _height(ingroup)
        out.length = _height(ingroup) + ingroup.length
        root = _Node()
        root.kids = [out, ingroup]
    else:
        root = _yule(rng, n_species)
    root.length = 0.0
    order = _number(root, n_species)
    tot = sum(nd.length for nd in order if nd is not root)
    for nd in order:
        nd.length = float(np.float32(nd.length * total_length / tot))
    for nd in order:
        nd.name = ("sp%02d" % nd.id) if not nd.kids else ("n%02d" % nd.id)
    N = 2 * n_species - 1
    children = np.full((N, 2), -1, dtype=np.int32)
    dist = np.zeros(N, dtype=np.float64)
    names = [""] * N
    for nd in order:
        names[nd.id] = nd.name
        dist[nd.id] = nd.length
        if nd.kids:
            ids = sorted(k.id for k in nd.kids)
            children[nd.id] = ids
    return Tree(n_species, children, dist, names, _newick(root))


def make_rev_q(pi, exch) -> np.ndarray:
    """REV rate matrix Q_ij = s_ij pi_j, rows summing to zero, scaled to one
    expected substitution per unit time."""
    pi = np.asarray(pi, dtype=np.float64)
    R = np.zeros((4, 4))
    iu = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    for (i, j), s in zip(iu, exch):
        R[i, j] = R[j, i] = s
    Q = R * pi[None, :]
    np.fill_diagonal(Q, -Q.sum(1))
    Q /= -(pi * np.diag(Q)).sum()
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(1))
    return Q


def _pmatrices(Q: np.ndarray, t: np.ndarray) -> np.ndarray:
    """P(t) = expm(Q t) for a batch of times t (any shape) -> [..., 4, 4]."""
    lam, V = np.linalg.eig(Q)
    lam = lam.real
    V = V.real
    Vi = np.linalg.inv(V)
    e = np.exp(lam * t[..., None])
    P = np.einsum("ij,...j,jk->...ik", V, e, Vi)
    return np.clip(P, 0.0, None)


def pick_clades(tree: Tree, sizes: List[int], seed: int, exclude_root_child: Optional[int] = None) -> List[int]:
    """Disjoint clades (internal nodes) with the given leaf counts, inside the ingroup."""
    rng = np.random.default_rng(seed)
    S = tree.n_species
    N = tree.n_nodes
    by_size = {}
    for v in range(S, N - 1):
        if v == exclude_root_child:
            continue
        by_size.setdefault(len(tree.leaves_under(v)), []).append(v)
    chosen: List[int] = []
    used = set()
    for k in sizes:
        cands = [v for v in by_size.get(k, []) if not (set(tree.nodes_under(v)) & used)]
        if not cands:
            # fall back to any clade of size in [2, k+1] that is still free
            cands = [v for sz in sorted(by_size) if 2 <= sz <= k + 1 for v in by_size[sz]
                     if not (set(tree.nodes_under(v)) & used)]
        v = int(cands[int(rng.integers(len(cands)))])
        chosen.append(v)
        used |= set(tree.nodes_under(v))
    return chosen


def simulate(tree: Tree, Q: np.ndarray, pi: np.ndarray, lengths: np.ndarray, branch_rate: np.ndarray,
             seed: int) -> np.ndarray:
    """Simulate all elements at once.  branch_rate: [E, N] per-branch rate
    multipliers.  Returns codes [S, total_columns] in 0..3 (a, c, g, t)."""
    rng = np.random.default_rng(seed)
    E = len(lengths)
    N = tree.n_nodes
    tot = int(lengths.sum())
    eidx = np.repeat(np.arange(E), lengths)
    states = np.zeros((N, tot), dtype=np.int8)
    root = N - 1
    cum_pi = np.cumsum(pi)
    states[root] = np.searchsorted(cum_pi, rng.random(tot) * cum_pi[-1], side="right").clip(0, 3)
    par = tree.parent()
    order = list(range(N - 2, -1, -1))  # parents have larger ids (postorder numbering)
    for v in order:
        p = par[v]
        P = _pmatrices(Q, branch_rate[:, v] * tree.distances[v])  # [E, 4, 4]
        cum = np.cumsum(P, axis=2)
        cum /= cum[:, :, 3:4]
        cp = cum[eidx, states[p]]  # [tot, 4]
        u = rng.random(tot)
        states[v] = (u[:, None] > cp).sum(1).clip(0, 3)
    return states[:tree.n_species]


def make_dataset(kind: str, n_elements: Optional[int] = None, seed: int = 0) -> Dataset:
    """kind: 'st12'  — 12 taxa, one outgroup, total length 1.2, 100 elements of
                       U{100..300} bp, 80 conserved (r1 = 0.35) and 20 accelerated
                       (r2 = 2.5) on a 3-taxon target clade, 5% '-' and 1% 'N';
             'st43'  — 43 taxa, total length 2.5, 8 targets in 3 clades, 5,000
                       elements of log-normal length (median 250, sigma 0.6,
                       clipped 50..2000), 10% accelerated with r2 ~ U[1.5, 4],
                       r1 ~ U[0.2, 0.6], 5% of (taxon, element) pairs missing
                       and 3% gap cells;
             'st43_stress' — underflow stress set: the st43 tree with all branch
                       lengths x5, 1,000 elements of 2,000 bp, r2 = 6;
             'st43_serve' — st43 with lengths clipped 50..5000;
             'gbgc120' — the gBGC model's workload: 120 taxa, total length 4.0,
                       20 targets in 6 clades, 20,000 elements of log-normal
                       length (median 300, sigma 0.6, clipped 50..3000), each
                       with a GC-bias strength B ~ Gamma(2, 1) on a random 20%
                       of its branches, selection -2 (conserved) everywhere but
                       the target clades of the 10% accelerated elements
                       (selection 0); sequences simulated under the
                       non-reversible rate matrix getRate(Q0, s, b) of
                       PhyloAcc-ST-GBGC (bpp_c.cpp:13-30); 3% gap cells and 5%
                       of (taxon, element) pairs missing, written with '*', the
                       model's gap character."""
    rng = np.random.default_rng(seed + 1000)
    if kind == "st12":
        S, total, E = 12, 1.2, 100 if n_elements is None else n_elements
        tree = make_tree(S, total, seed)
        exch = rng.uniform(0.5, 2.0, 6)
        pi = np.array([0.30, 0.20, 0.20, 0.30])
        ingroup_root = int(tree.children[-1][1]) if tree.children[-1][1] >= S else int(tree.children[-1][0])
        clades = pick_clades(tree, [3], seed, exclude_root_child=ingroup_root)
        lengths = rng.integers(100, 301, size=E).astype(np.int32)
        accel = np.zeros(E, bool)
        accel[np.arange(E) >= int(round(0.8 * E))] = True
        r1 = np.full(E, 0.35)
        r2 = np.where(accel, 2.5, 0.0)
        miss_pairs = 0.0
        gap_p, n_p = 0.05, 0.01
    elif kind in ("st43", "st43_stress", "st43_serve"):
        S, total = 43, 2.5
        E = (1000 if kind == "st43_stress" else (200000 if kind == "st43_serve" else 5000)) \
            if n_elements is None else n_elements
        tree = make_tree(S, total, seed)
        if kind == "st43_stress":
            tree.distances = (tree.distances * 5).astype(np.float32).astype(np.float64)
        exch = rng.uniform(0.5, 2.0, 6)
        pi = np.array([0.30, 0.20, 0.20, 0.30])
        ingroup_root = int(tree.children[-1][1]) if tree.children[-1][1] >= S else int(tree.children[-1][0])
        clades = pick_clades(tree, [3, 3, 2], seed, exclude_root_child=ingroup_root)
        if kind == "st43_stress":
            lengths = np.full(E, 2000, dtype=np.int32)
        else:
            hi = 5000 if kind == "st43_serve" else 2000
            lengths = np.clip(np.rint(np.exp(np.log(250) + 0.6 * rng.standard_normal(E))), 50, hi).astype(np.int32)
        accel = rng.random(E) < 0.10
        r1 = rng.uniform(0.2, 0.6, E)
        r2 = np.where(accel, 6.0 if kind == "st43_stress" else rng.uniform(1.5, 4.0, E), 0.0)
        miss_pairs = 0.05
        gap_p, n_p = 0.03, 0.0
    elif kind == "gbgc120":
        return _make_gbgc(20000 if n_elements is None else n_elements, seed, rng)
    else:
        raise ValueError(kind)
    Q = make_rev_q(pi, exch)
    N = tree.n_nodes
    target_nodes = set()
    for c in clades:
        target_nodes |= set(tree.nodes_under(c))
    target_leaves = sorted(v for v in target_nodes if v < S)
    br = np.repeat(r1[:, None], N, axis=1)
    tmask = np.zeros(N, bool)
    tmask[list(target_nodes)] = True
    br[np.ix_(accel, tmask)] = r2[accel][:, None]
    codes = simulate(tree, Q, pi, lengths, br, seed + 7)
    chars = BASES[codes]  # [S, tot]
    tot = chars.shape[1]
    u = rng.random((S, tot))
    chars = np.where(u < gap_p, np.uint8(ord("-")), chars)
    if n_p > 0:
        chars = np.where((u >= gap_p) & (u < gap_p + n_p), np.uint8(ord("n")), chars)
    starts = np.zeros(E + 1, dtype=np.int64)
    starts[1:] = np.cumsum(lengths)
    if miss_pairs > 0:
        mp = rng.random((E, S)) < miss_pairs
        for e, s in zip(*np.nonzero(mp)):
            chars[s, starts[e]:starts[e + 1]] = ord("-")
    # per-element blocks S x GG
    offsets = np.zeros(E, dtype=np.int64)
    offsets[1:] = np.cumsum(lengths[:-1].astype(np.int64) * S)
    blocks = np.empty(int(lengths.sum()) * S, dtype=np.uint8)
    for e in range(E):
        blk = chars[:, starts[e]:starts[e + 1]]
        blocks[offsets[e]:offsets[e] + blk.size] = blk.reshape(-1)
    outgroup = [0] if tree.children[-1][0] == 0 else [int(tree.children[-1][0])]
    outgroup = [v for v in outgroup if v < S]
    conserve = [s for s in range(S) if s not in target_leaves and s not in outgroup]
    names = ["elem%05d" % e for e in range(E)]
    return Dataset(tree, pi, Q, outgroup, conserve, target_leaves, lengths, offsets, blocks, names, accel, r1, r2)


def gbgc_rate(Q0: np.ndarray, s: float, b: float) -> np.ndarray:
    """getRate of PhyloAcc-ST-GBGC (bpp_c.cpp:13-30): Q0 scaled entrywise by
    f(s + b B_ij), f(x) = x / (1 - e^-x), B = +1 from A/T to C/G, -1 back."""
    if s == 0 and b == 0:
        return Q0.copy()
    weak = np.array([1, 0, 0, 1], bool)
    B = np.where(weak[:, None] & ~weak[None, :], b, np.where(~weak[:, None] & weak[None, :], -b, 0.0)) + s
    with np.errstate(divide="ignore", invalid="ignore"):
        F = np.where(B == 0, 1.0, B / (1 - np.exp(-B)))
    Q = Q0 * F
    Q[np.diag_indices(4)] -= Q.sum(1)
    return Q


def _make_gbgc(E: int, seed: int, rng) -> Dataset:
    S, total = 120, 4.0
    tree = make_tree(S, total, seed)
    N = tree.n_nodes
    exch = rng.uniform(0.5, 2.0, 6)
    pi = np.array([0.30, 0.20, 0.20, 0.30])
    Q0 = make_rev_q(pi, exch)
    ingroup_root = int(tree.children[-1][1]) if tree.children[-1][1] >= S else int(tree.children[-1][0])
    clades = pick_clades(tree, [4, 4, 3, 3, 3, 3], seed, exclude_root_child=ingroup_root)
    target_nodes = set()
    for c in clades:
        target_nodes |= set(tree.nodes_under(c))
    target_leaves = sorted(v for v in target_nodes if v < S)
    tmask = np.zeros(N, bool)
    tmask[list(target_nodes)] = True
    lengths = np.clip(np.rint(np.exp(np.log(300) + 0.6 * rng.standard_normal(E))), 50, 3000).astype(np.int32)
    accel = rng.random(E) < 0.10
    bstr = rng.gamma(2.0, 1.0, E)
    bflag = rng.random((E, N)) < 0.2
    # per element, the four rate matrices (selection -2 / 0) x (no bias / bias)
    Qs = np.empty((E, 4, 4, 4))
    for e in range(E):
        for k, (sv, bv) in enumerate(((-2.0, 0.0), (0.0, 0.0), (-2.0, bstr[e]), (0.0, bstr[e]))):
            Qs[e, k] = gbgc_rate(Q0, sv, bv)
    lam, V = np.linalg.eig(Qs)
    Vi = np.linalg.inv(V)
    tot = int(lengths.sum())
    eidx = np.repeat(np.arange(E), lengths)
    srng = np.random.default_rng(seed + 7)
    states = np.zeros((N, tot), dtype=np.int8)
    cum_pi = np.cumsum(pi)
    states[N - 1] = np.searchsorted(cum_pi, srng.random(tot) * cum_pi[-1], side="right").clip(0, 3)
    par = tree.parent()
    for v in range(N - 2, -1, -1):
        k = np.where(accel & tmask[v], 1, 0) + np.where(bflag[:, v], 2, 0)
        ar = np.arange(E)
        ex = np.exp(lam[ar, k] * tree.distances[v])
        P = np.einsum("eij,ej,ejk->eik", V[ar, k], ex, Vi[ar, k]).real.clip(0.0, None)
        cum = np.cumsum(P, axis=2)
        cum /= cum[:, :, 3:4]
        cp = cum[eidx, states[par[v]]]
        states[v] = (srng.random(tot)[:, None] > cp).sum(1).clip(0, 3)
    chars = BASES[states[:S]]
    u = rng.random((S, tot))
    star = np.uint8(ord("*"))
    chars = np.where(u < 0.03, star, chars)
    starts = np.zeros(E + 1, dtype=np.int64)
    starts[1:] = np.cumsum(lengths)
    mp = rng.random((E, S)) < 0.05
    for e, sp in zip(*np.nonzero(mp)):
        chars[sp, starts[e]:starts[e + 1]] = star
    offsets = np.zeros(E, dtype=np.int64)
    offsets[1:] = np.cumsum(lengths[:-1].astype(np.int64) * S)
    blocks = np.empty(int(lengths.sum()) * S, dtype=np.uint8)
    for e in range(E):
        blocks[offsets[e]:offsets[e] + S * int(lengths[e])] = chars[:, starts[e]:starts[e + 1]].reshape(-1)
    outgroup = [0] if tree.children[-1][0] == 0 else [int(tree.children[-1][0])]
    outgroup = [v for v in outgroup if v < S]
    conserve = [s for s in range(S) if s not in target_leaves and s not in outgroup]
    names = ["elem%05d" % e for e in range(E)]
    return Dataset(tree, pi, Q0, outgroup, conserve, target_leaves, lengths, offsets, blocks, names, accel,
                   np.full(E, -2.0), np.where(accel, 0.0, -2.0))


# ---------------------------------------------------------------------------
# PhyloAcc-ST input files
# ---------------------------------------------------------------------------
def write_mod(ds: Dataset, path: str) -> None:
    with open(path, "w") as f:
        f.write("ALPHABET: A C G T\nORDER: 0\nSUBST_MOD: REV\n")
        f.write("BACKGROUND: " + " ".join(repr(float(x)) for x in ds.pi) + "\n")
        f.write("RATE_MAT:\n")
        for i in range(4):
            f.write("  " + " ".join(repr(float(x)) for x in ds.Q[i]) + "\n")
        f.write("TREE: " + ds.tree.newick + "\n")


def write_inputs(ds: Dataset, outdir: str, prefix: str = "synth", burnin: int = 500, mcmc: int = 1000,
                 seed: int = 0, extra: Optional[dict] = None, species_order=None) -> str:
    """Write .mod, FASTA, bed and a PhyloAcc-ST cfg.  Returns the cfg path."""
    os.makedirs(outdir, exist_ok=True)
    S = ds.tree.n_species
    mod = os.path.join(outdir, prefix + ".mod")
    fa = os.path.join(outdir, prefix + ".fa")
    bed = os.path.join(outdir, prefix + ".bed")
    write_mod(ds, mod)
    rows = [[] for _ in range(S)]
    for e in range(ds.n_elements):
        blk = ds.element(e)
        for s in range(S):
            rows[s].append(blk[s].tobytes())
    order = list(range(S)) if species_order is None else list(species_order)
    with open(fa, "w") as f:
        for s in order:
            seq = b"".join(rows[s]).decode().upper()
            f.write(">" + ds.tree.names[s] + "\n")
            for i in range(0, len(seq), 80):
                f.write(seq[i:i + 80] + "\n")
    with open(bed, "w") as f:
        pos = 0
        for e in range(ds.n_elements):
            L = int(ds.lengths[e])
            f.write("%s\t%d\t%d\n" % (ds.element_names[e], pos, pos + L))
            pos += L
    res = os.path.join(outdir, "out")
    os.makedirs(res, exist_ok=True)
    cfg = os.path.join(outdir, prefix + ".cfg")
    names = ds.tree.names
    kv = {
        "PHYTREE_FILE": mod, "SEG_FILE": bed, "ALIGN_FILE": fa, "RESULT_FOLDER": res, "PREFIX": prefix,
        "BURNIN": burnin, "MCMC": mcmc, "CHAIN": 1, "SEED": seed,
        "TARGETSPECIES": ";".join(names[s] for s in ds.target),
        "OUTGROUP": ";".join(names[s] for s in ds.outgroup),
        "CONSERVE": ";".join(names[s] for s in ds.conserve),
        "NUM_THREAD": 1,
    }
    if extra:
        kv.update(extra)
    with open(cfg, "w") as f:
        for k, v in kv.items():
            f.write("%s %s\n" % (k, v))
    return cfg
