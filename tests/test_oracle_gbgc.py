"""The oracle's restatement of the gBGC model's likelihood engine
(oracle/oracle_gbgc.cpp) against what the unmodified gBGC reference computes
from the same inputs and states (tests/golden/gbgc_engine/engine.npz, written
by tests/golden/make_gbgc_engine_golden.py): the six per-branch log
transition matrices, per-column log-likelihoods and expected base-pair
counts, for three random (Z, B, selection, bias) states on each element of
the gbgc12_default case."""
import os

import numpy as np

from golden_io import GOLDEN, load_case
from oracle import pyoracle as po


def _records():
    d = np.load(os.path.join(GOLDEN, "gbgc_engine", "engine.npz"))
    n = int(d["n_records"])
    return [{k[len("r%d_" % i):]: d[k] for k in d.files if k.startswith("r%d_" % i)} for i in range(n)]


def test_gbgc_engine_matches_reference(built):
    ds, _, _ = load_case("gbgc12_default")
    recs = _records()
    assert len(recs) == 12
    N = ds.tree.n_nodes
    for r in recs:
        e = int(r["element"])
        z = r["Z"].astype(np.int32)
        b = r["B"].astype(np.int32)
        got = po.gbgc_engine(ds, e, z, b, float(r["sc"]), float(r["sn"]), float(r["gb"]))
        assert got["filtered"] == 0
        assert got["root"] == int(r["root"])
        assert (got["missing"] == r["missing"].astype(np.uint8)).all()
        nodes = r["nodes"].astype(int)
        for k in range(6):
            want = r["logP%d" % k].reshape(N, 4, 4)
            for s in nodes[:-1]:
                if r["missing"][s]:
                    continue
                np.testing.assert_allclose(got["logp"][k, s], want[s], rtol=1e-12, atol=1e-13)
        np.testing.assert_allclose(got["col"], r["col"], rtol=1e-12, atol=0)
        np.testing.assert_allclose(got["counts"], r["counts"].reshape(N, 4, 4), rtol=1e-10, atol=1e-12)


def test_gbgc_rate_spectrum_is_real_and_matches_pade(built):
    """Q(s, b) = getRate(Q0, s, b) (bpp_c.cpp:13-30) satisfies detailed balance
    with pi'_i = pi_i h(i), h taking one value on A/T and another on C/G
    (f(x) / f(-x) = e^x for f(x) = x / (1 - e^-x)), so its spectrum is real and
    the reference's real part of eig_gen loses nothing.  Checked over a grid
    of selection and bias values: eigenvalues real, detailed balance holds, and
    the oracle's eigen-based log P (as the reference computes it) equals
    log(expm(Q d)^T) from scipy's Padé scaling-and-squaring to 1e-11."""
    from scipy.linalg import expm
    from phyloacc_gb300 import synth
    ds, _, _ = load_case("gbgc12_default")
    Q0 = np.array(ds.Q, dtype=float)
    N = ds.tree.n_nodes
    e = 0
    GG = int(ds.lengths[e])
    for s in (-5.0, -2.0, -0.3, 0.0, 0.7, 3.0):
        for b in (0.0, 0.5, 3.0, 9.0):
            Q = synth.gbgc_rate(Q0, s, b)
            lam = np.linalg.eigvals(Q)
            assert np.abs(lam.imag).max() < 1e-10 * np.abs(lam).max()
            # detailed balance with the stationary distribution of Q
            w, V = np.linalg.eig(Q.T)
            pi = np.real(V[:, np.argmin(np.abs(w))])
            pi = pi / pi.sum()
            F = pi[:, None] * Q
            np.testing.assert_allclose(F, F.T, rtol=1e-10, atol=1e-13)
            # the oracle's class matrices at this (s, b): class 4 is cons + B
            z = np.ones(N, np.int32)
            bf = np.ones(N, np.int32)
            got = po.gbgc_engine(ds, e, z, bf, s, 1.0, b)
            ok = 0
            for node in range(N - 1):
                if not np.any(got["logp"][4, node]):
                    continue
                d = float(ds.tree.distances[node])
                if node in np.flatnonzero(got["missing"]):
                    continue
                want = np.log(expm(Q * d).T)
                np.testing.assert_allclose(got["logp"][4, node], want, rtol=1e-11, atol=1e-11)
                ok += 1
            assert ok > 0
