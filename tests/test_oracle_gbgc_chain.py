"""The oracle's gBGC chain (oracle/oracle_gbgc.cpp, oracle_gbgc_run_element)
against what the unmodified gBGC reference wrote for the gbgc12_default case
(tests/golden/gbgc12_default) and the gbgc43_missing case (43 taxa with the
outgroup, three conserved leaves and a target leaf missing in some elements): the per-iteration traces of the three models
(full log-likelihood, selection, GC bias, B and Z on every node), the
element table (Eval2's marginal likelihoods and the best full
log-likelihoods) and the per-model tables of rate medians and B / Z
frequencies.  The reference prints 8 significant digits in the traces and
element table and 6 in the per-model tables; the comparisons allow those."""
import os

import numpy as np
import pytest

from golden_io import GOLDEN, as_float, load_case, read_table
from oracle import pyoracle as po
from phyloacc_gb300 import abi


# cfg keys of the gBGC program (src/PhyloAcc-ST-GBGC/SRC/main.cpp:83-259) -> option fields
GBGC_KEYS = {"CONSERVE_RATE": "conserve_rate", "ACCE_RATE": "acce_rate",
             "CONSERVE_PRIOR_A": "conserve_prior_a", "CONSERVE_PRIOR_B": "conserve_prior_b",
             "ACCE_PRIOR_A": "acce_prior_a", "ACCE_PRIOR_B": "acce_prior_b",
             "PREP_LRATE": "prep_lrate", "PREP_GRATE": "prep_grate", "CONSTOMIS": "cons_to_mis",
             "GAP_PROP": "missing_thres", "CONSERVE_PROP": "conserve_prop"}


def gbgc_opts(ds, kv):
    o = abi.gbgc_default_opts(ds.target)
    o.burnin, o.mcmc, o.seed = int(kv["BURNIN"]), int(kv["MCMC"]), int(kv["SEED"])
    if "GAPCHAR" in kv:
        o.gapchar = ord(kv["GAPCHAR"][0])
    for k, f in GBGC_KEYS.items():
        if k in kv:
            setattr(o, f, float(kv[k]))
    return o


def _runs(case):
    ds, _, kv = load_case(case)
    o = gbgc_opts(ds, kv)
    return ds, o, [po.gbgc_run(ds, o, e) for e in range(ds.n_elements)]


CASES = ["gbgc12_default", "gbgc43_missing", "gbgc12_options", "gbgc43_dash"]


@pytest.mark.parametrize("case", CASES)
def test_gbgc_chain_traces_match_reference(built, case):
    ds, o, runs = _runs(case)
    tr = np.load(os.path.join(GOLDEN, case, "traces.npz"))
    for e, r in enumerate(runs):
        assert r["status"] == abi.PACC_OK
        for m in range(3):
            want = tr["%d_%d" % (m, e)]
            got = r["trace"][m]
            assert got.shape == want.shape
            np.testing.assert_allclose(got, want, rtol=1e-7, atol=1e-9)


@pytest.mark.parametrize("case", CASES)
def test_gbgc_chain_tables_match_reference(built, case):
    ds, o, runs = _runs(case)
    N = ds.tree.n_nodes
    out = os.path.join(GOLDEN, case, "out")
    hdr, rows = read_table(os.path.join(out, "case_elem_lik.txt"))
    assert hdr[2:] == ["loglik_NUll", "loglik_RES", "loglik_all", "log_ratio", "loglik_Max1", "loglik_Max2",
                       "loglik_Max3"]
    for e, (r, row) in enumerate(zip(runs, rows)):
        got = [r["loglik_null"], r["loglik_res"], r["loglik_all"], r["loglik_res"] - r["loglik_null"]] + \
            list(r["max_loglik"])
        np.testing.assert_allclose(got, [as_float(x) for x in row[2:9]], rtol=1e-7, atol=1e-6)
    for m in range(3):
        _, rows = read_table(os.path.join(out, "case_rate_postZ_%d.txt" % m))
        for e, (r, row) in enumerate(zip(runs, rows)):
            vals = [as_float(x) for x in row[1:] if x != ""]
            got = list(r["rates"][m]) + list(r["post_b"][m]) + list(r["post_z"][m].reshape(-1))
            assert len(vals) == 3 + N + 4 * N
            np.testing.assert_allclose(got, vals, rtol=1e-5, atol=1e-6)
    # Max_Z of the full model (the _1_elem_Z table)
    lines = [ln.rstrip("\n\t").split("\t") for ln in open(os.path.join(out, "case_1_elem_Z.txt"))][1:]
    for r, ln in zip(runs, lines):
        assert [int(x) for x in ln] == list(r["max_z"][1])


def test_gbgc_chain_two_chains_match_reference(built):
    """CHAIN 2 (gbgc43_chain2): the second chain starts every node from Z = 0
    (bpp.cur_Z, never written without SAMPLE_HYPER), which changes the traces
    and Z frequencies of the nodes off the element's tree (element 1 lost its
    outgroup, so its root moved); both chains' traces and every table the
    reference wrote (rate_postZ rows of both chains, the last chain's
    elem_lik and 1_elem_Z)."""
    case = "gbgc43_chain2"
    ds, _, kv = load_case(case)
    N = ds.tree.n_nodes
    tr = np.load(os.path.join(GOLDEN, case, "traces.npz"))
    runs = []
    for k in range(2):
        o = gbgc_opts(ds, kv)
        o.chain = k
        runs.append([po.gbgc_run(ds, o, e) for e in range(ds.n_elements)])
        for e, r in enumerate(runs[k]):
            for m in range(3):
                want = tr["%d_%d" % (m, e) + ("_c1" if k else "")]
                np.testing.assert_allclose(r["trace"][m], want, rtol=1e-7, atol=1e-9, err_msg="%d %d %d" % (k, e, m))
    assert not np.array_equal(runs[0][1]["post_z"], runs[1][1]["post_z"])   # the off-tree nodes differ
    out = os.path.join(GOLDEN, case, "out")
    for m in range(3):
        _, rows = read_table(os.path.join(out, "case_rate_postZ_%d.txt" % m))
        assert len(rows) == 2 * ds.n_elements
        for i, row in enumerate(rows):
            r = runs[i // ds.n_elements][i % ds.n_elements]
            vals = [as_float(x) for x in row[1:] if x != ""]
            got = list(r["rates"][m]) + list(r["post_b"][m]) + list(r["post_z"][m].reshape(-1))
            np.testing.assert_allclose(got, vals, rtol=1e-5, atol=1e-6)
    _, rows = read_table(os.path.join(out, "case_elem_lik.txt"))
    for r, row in zip(runs[1], rows):
        got = [r["loglik_null"], r["loglik_res"], r["loglik_all"]]
        np.testing.assert_allclose(got, [as_float(x) for x in row[2:5]], rtol=1e-7, atol=1e-6)
