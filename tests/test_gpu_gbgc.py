"""The gBGC model's likelihood engine on the GPU (pacc_gbgc_engine) against
the unmodified gBGC reference's own numbers (tests/golden/gbgc_engine) and
against the oracle's restatement (oracle/oracle_gbgc.cpp) on larger inputs.

Tolerances.  The device builds P = exp(Q d) by Padé scaling and squaring, the
reference by an eigendecomposition: both are FP64 and agree to a few units in
the last place of P's larger entries, so log P is compared with rtol 1e-9
(absolute 1e-10) and P itself with absolute 1e-13.  With FP64 partials the
per-column log-likelihoods agree to 1e-10 relative and the expected counts to
1e-9 relative (absolute 1e-9).  With FP32 partials (FP64 matrices and sums)
a column's log-likelihood is within 2e-6 x max(1, |value|) and a count within
1e-4 relative plus 1e-5 x columns absolute."""
import os

import numpy as np
import pytest

from golden_io import GOLDEN, load_case
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _records():
    d = np.load(os.path.join(GOLDEN, "gbgc_engine", "engine.npz"))
    n = int(d["n_records"])
    return [{k[len("r%d_" % i):]: d[k] for k in d.files if k.startswith("r%d_" % i)} for i in range(n)]


def _ctx(ds, precision):
    from phyloacc_gb300 import Context, abi
    o = abi.default_opts()
    o.precision = precision
    return Context(ds, o)


def _check(got, want_logp, want_col, want_counts, nodes, missing, GG, fp32):
    for s in nodes[:-1]:
        if missing[s]:
            continue
        for k in range(6):
            w = want_logp[k, s]
            if not np.any(w):            # a class the reference does not build on this branch
                assert not np.any(got["logp"][k, s])
                continue
            np.testing.assert_allclose(got["logp"][k, s], w, rtol=1e-9, atol=1e-10)
            np.testing.assert_allclose(np.exp(got["logp"][k, s]), np.exp(w), rtol=0, atol=1e-13)
    if fp32:
        err = np.abs(got["col"] - want_col) / np.maximum(1.0, np.abs(want_col))
        assert err.max() <= 2e-6, err.max()
        np.testing.assert_allclose(got["counts"], want_counts, rtol=1e-4, atol=1e-5 * GG)
    else:
        np.testing.assert_allclose(got["col"], want_col, rtol=1e-10, atol=0)
        np.testing.assert_allclose(got["counts"], want_counts, rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_gbgc_engine_matches_reference_golden(built, precision):
    ds, _, _ = load_case("gbgc12_default")
    ctx = _ctx(ds, precision)
    N = ds.tree.n_nodes
    for r in _records():
        e = int(r["element"])
        got = ctx.gbgc_engine(e, r["Z"], r["B"], float(r["sc"]), float(r["sn"]), float(r["gb"]))
        assert got["filtered"] == 0
        assert got["root"] == int(r["root"])
        assert (got["missing"] == r["missing"].astype(np.uint8)).all()
        want_logp = np.stack([r["logP%d" % k].reshape(N, 4, 4) for k in range(6)])
        _check(got, want_logp, r["col"], r["counts"].reshape(N, 4, 4), r["nodes"].astype(int),
               r["missing"], int(r["GG"]), precision == 1)


def _random_state(rng, ds, o):
    N = ds.tree.n_nodes
    z = rng.integers(0, 3, N).astype(np.int32)
    b = (rng.random(N) < 0.35).astype(np.int32)
    return z, b


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_gbgc_engine_matches_oracle_st43(built, precision):
    """43 taxa, 40 elements of 150-1500 columns with gaps ('-' as the gap
    character, so that taxa go missing and the outgroup path collapses), one
    random state per element; the outgroup path takes Z in {0, 1} as the
    model allows."""
    from phyloacc_gb300 import synth
    ds = synth.make_dataset("st43", n_elements=40, seed=7)
    ctx = _ctx(ds, precision)
    rng = np.random.default_rng(11)
    n_run = n_filtered = 0
    for e in range(ds.n_elements):
        z, b = _random_state(rng, ds, None)
        sc, sn, gb = -0.5 - 2.5 * rng.random(), -1.0 + 3.0 * rng.random(), 0.1 + 2.9 * rng.random()
        ref = po.gbgc_engine(ds, e, z, b, sc, sn, gb, gapchar="-")
        if ref["filtered"]:
            got = ctx.gbgc_engine(e, z, b, sc, sn, gb, gapchar="-")
            assert got["filtered"] == 1
            n_filtered += 1
            continue
        # no accelerated class on the outgroup path: redraw those nodes in {0, 1}
        fixed = np.all(ref["logp"][2] == 0, axis=(1, 2)) & ~ref["missing"].astype(bool)
        z[fixed & (z == 2)] = rng.integers(0, 2, int((fixed & (z == 2)).sum()))
        ref = po.gbgc_engine(ds, e, z, b, sc, sn, gb, gapchar="-")
        got = ctx.gbgc_engine(e, z, b, sc, sn, gb, gapchar="-")
        assert got["root"] == ref["root"]
        assert (got["missing"] == ref["missing"]).all()
        nodes = _postorder(ds, ref)
        _check(got, ref["logp"], ref["col"], ref["counts"], nodes, ref["missing"], int(ds.lengths[e]), precision == 1)
        n_run += 1
    assert n_run >= 30


def _postorder(ds, ref):
    """Nodes on which the oracle built matrices, then the root (the order does
    not matter to the checks)."""
    N = ds.tree.n_nodes
    built_ = [s for s in range(N) if np.any(ref["logp"][0, s])]
    return built_ + [ref["root"]]


def test_gbgc_engine_rejects_accelerated_outgroup_path(built):
    ds, _, _ = load_case("gbgc12_default")
    ctx = _ctx(ds, 0)
    r = _records()[0]
    z = r["Z"].copy()
    N = ds.tree.n_nodes
    want0 = r["logP2"].reshape(N, 4, 4)
    nodes = r["nodes"].astype(int)
    fixed = [s for s in nodes[:-1] if not r["missing"][s] and not np.any(want0[s])]
    assert fixed
    z[fixed[0]] = 2
    from phyloacc_gb300 import PaccError
    with pytest.raises(PaccError):
        ctx.gbgc_engine(int(r["element"]), z, r["B"], float(r["sc"]), float(r["sn"]), float(r["gb"]))
