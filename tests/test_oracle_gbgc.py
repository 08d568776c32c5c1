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
