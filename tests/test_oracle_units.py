"""Known-answer and distribution tests that pin the oracle's building blocks:
the Philox generator (published Random123 known-answer vectors), the samplers
(against scipy.stats), the eigendecomposition (against scipy.linalg.expm) and
the pruning likelihood (against brute-force enumeration of internal states)."""
import itertools

import numpy as np
import pytest
import scipy.linalg as sl
import scipy.stats as ss

from oracle import pyoracle as po
from phyloacc_gb300 import abi, synth


def test_philox_known_answers():
    # Salmon et al. (SC'11), Random123 kat_vectors for philox4x32-10
    assert po.philox([0, 0, 0, 0], [0, 0]).tolist() == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert po.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2).tolist() == [0x408F276D, 0x41C83B0E, 0xA20BC7C6,
                                                                       0x6D5451FD]
    assert po.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]).tolist() == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_stream_layout():
    w = po.stream(11, 0, 16)
    for b in range(4):
        assert (w[4 * b:4 * b + 4] == po.philox([b, 0, 0, 0], [11, 0])).all()
    assert (po.stream(11, 5, 7) == w[5:12]).all()


@pytest.mark.parametrize("a,b", [(10.0, 0.2), (5.0, 0.04), (0.4, 2.0), (33.0, 0.03)])
def test_gamma_sampler(a, b):
    x = po.sample_gamma(3, a, b, 20000)
    assert ss.kstest(x, ss.gamma(a, scale=b).cdf).pvalue > 1e-3


@pytest.mark.parametrize("a,b", [(4.0, 1.0), (1.0, 9.0), (0.5, 0.5)])
def test_beta_sampler(a, b):
    x = po.sample_beta(5, a, b, 20000)
    assert ss.kstest(x, ss.beta(a, b).cdf).pvalue > 1e-3


def test_categorical_sampler():
    p = np.array([0.1, 0.0, 2.5, 1.4])
    x = po.sample_categorical(9, p, 40000)
    counts = np.bincount(x, minlength=4)
    assert counts[1] == 0
    exp = p / p.sum() * len(x)
    keep = exp > 0
    assert ss.chisquare(counts[keep], exp[keep]).pvalue > 1e-3


def _rand_rev(rng):
    pi = rng.dirichlet([5, 5, 5, 5])
    return synth.make_rev_q(pi, rng.uniform(0.3, 3.0, 6)), pi


def test_eigen_matches_expm():
    rng = np.random.default_rng(0)
    for _ in range(20):
        Q, _ = _rand_rev(rng)
        st, lam, V, Vi = po.eigen(Q)
        assert st == 0
        for t in (0.01, 0.3, 2.0, 7.0):
            P = V @ np.diag(np.exp(lam * t)) @ Vi
            assert np.abs(P - sl.expm(Q * t)).max() < 1e-13


def test_eigen_repeated_spectrum():
    # JC69: eigenvalue -4/3 with multiplicity 3
    Q = np.full((4, 4), 1.0 / 3.0)
    np.fill_diagonal(Q, -1.0)
    st, lam, V, Vi = po.eigen(Q)
    assert st == 0
    P = V @ np.diag(np.exp(lam * 0.7)) @ Vi
    assert np.abs(P - sl.expm(Q * 0.7)).max() < 1e-13


def _tiny_dataset(S, seed):
    ds = synth.make_dataset("st12", n_elements=3, seed=seed)
    t = synth.make_tree(S, 0.9, seed)
    rng = np.random.default_rng(seed)
    Q, pi = _rand_rev(rng)
    L = 60
    E = 2
    chars = np.frombuffer(b"acgtn-ry", np.uint8)
    bases = chars[rng.choice(8, size=E * S * L, p=[.22, .22, .22, .22, .03, .03, .03, .03])]
    return synth.Dataset(t, pi, Q, [0], list(range(1, S)), [], np.full(E, L, np.int32),
                         np.arange(E, dtype=np.int64) * S * L, bases.astype(np.uint8), ["a", "b"],
                         np.zeros(E, bool), np.zeros(E), np.zeros(E))


def _brute_force_column(ds, col_codes, z, rc, rn):
    """Sum over all internal-node states of pi(root) prod P(parent -> child)."""
    t = ds.tree
    S, N = t.n_species, t.n_nodes
    lam, V = np.linalg.eig(ds.Q)
    rates = {0: 1.0, 1: rc, 2: rn}
    P = {}
    par = t.parent()
    for v in range(N - 1):
        P[v] = sl.expm(ds.Q * t.distances[v] * rates[int(z[v])])
    masks = {ord("a"): [0], ord("c"): [1], ord("g"): [2], ord("t"): [3], ord("r"): [0, 2], ord("y"): [1, 3]}
    total = 0.0
    internal = list(range(S, N))
    for states in itertools.product(range(4), repeat=len(internal)):
        st = dict(zip(internal, states))
        w = ds.pi[st[N - 1]]
        for v in internal[:-1]:
            w *= P[v][st[par[v]], st[v]]
        for s in range(S):
            allowed = masks.get(int(col_codes[s]))
            if allowed is None:
                continue  # gap / N: not included
            w *= sum(P[s][st[par[s]], b] for b in allowed)
        total += w
    return np.log(total)


@pytest.mark.parametrize("S", [3, 4, 5])
def test_loglik_brute_force(S):
    ds = _tiny_dataset(S, seed=S)
    o = abi.default_opts()
    rng = np.random.default_rng(S)
    for e in range(ds.n_elements):
        z = rng.integers(0, 3, ds.tree.n_nodes).astype(np.int32)
        ll = po.loglik(ds, o, e, z, 0.4, 2.0)
        blk = ds.element(e)
        for g in range(0, ds.lengths[e], 7):
            bf = _brute_force_column(ds, blk[:, g], z, 0.4, 2.0)
            # columns where every leaf is gap/N contribute log(sum pi)
            assert abs(ll[g] - bf) < 1e-12 * max(1.0, abs(bf)), (e, g, ll[g], bf)
