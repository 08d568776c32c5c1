"""The gBGC chain on the GPU (pacc_gbgc_run) against the unmodified gBGC
reference's traces and tables (tests/golden/gbgc12_default, gbgc43_missing)
and against the oracle's chain on larger inputs.

With FP64 partials the device follows the reference draw for draw: the
branch matrices come from Padé approximants instead of eigendecompositions
and the passes run in linear instead of log space, which moves the
log-likelihoods by about 1e-12 relative, far below what could flip an MH
decision in these chains; the traces are compared at the reference's 8 printed
digits (rtol 1e-7) and the tables as the oracle's test compares them.  With
FP32 partials the per-column log-likelihoods move by ~1e-6 relative, so the
chain leaves the reference's path at the first MH decision that close; that
leg checks the first iterations draw for draw and the element table within
Monte Carlo error."""
import os

import numpy as np
import pytest

from golden_io import GOLDEN, as_float, load_case, read_table
from test_oracle_gbgc_chain import gbgc_opts

pytestmark = pytest.mark.gpu

CASES = ["gbgc12_default", "gbgc43_missing", "gbgc12_options", "gbgc43_dash"]


def _ctx(ds, precision):
    from phyloacc_gb300 import Context, abi
    o = abi.default_opts()
    o.precision = precision
    return Context(ds, o)


@pytest.mark.parametrize("case", CASES)
def test_gbgc_chain_fp64_matches_reference(built, case):
    ds, _, kv = load_case(case)
    o = gbgc_opts(ds, kv)
    ctx = _ctx(ds, 0)
    runs = ctx.gbgc_run(o, trace=True)
    tr = np.load(os.path.join(GOLDEN, case, "traces.npz"))
    N = ds.tree.n_nodes
    for e, r in enumerate(runs):
        assert r["status"] == 0
        for m in range(3):
            want = tr["%d_%d" % (m, e)]
            np.testing.assert_allclose(r["trace"][m], want, rtol=1e-7, atol=1e-9,
                                       err_msg="element %d model %d" % (e, m))
    out = os.path.join(GOLDEN, case, "out")
    _, rows = read_table(os.path.join(out, "case_elem_lik.txt"))
    for r, row in zip(runs, rows):
        got = [r["loglik_null"], r["loglik_res"], r["loglik_all"], r["loglik_res"] - r["loglik_null"]] + \
            list(r["max_loglik"])
        np.testing.assert_allclose(got, [as_float(x) for x in row[2:9]], rtol=1e-7, atol=1e-6)
    for m in range(3):
        _, rows = read_table(os.path.join(out, "case_rate_postZ_%d.txt" % m))
        for r, row in zip(runs, rows):
            vals = [as_float(x) for x in row[1:] if x != ""]
            got = list(r["rates"][m]) + list(r["post_b"][m]) + list(r["post_z"][m].reshape(-1))
            assert len(vals) == 3 + N + 4 * N
            np.testing.assert_allclose(got, vals, rtol=1e-5, atol=1e-6)
    lines = [ln.rstrip("\n\t").split("\t") for ln in open(os.path.join(out, "case_1_elem_Z.txt"))][1:]
    for r, ln in zip(runs, lines):
        assert [int(x) for x in ln] == list(r["max_z"][1])


def test_gbgc_chain_fp32_follows_reference(built):
    ds, _, kv = load_case("gbgc12_default")
    o = gbgc_opts(ds, kv)
    runs = _ctx(ds, 1).gbgc_run(o, trace=True)
    tr = np.load(os.path.join(GOLDEN, "gbgc12_default", "traces.npz"))
    _, rows = read_table(os.path.join(GOLDEN, "gbgc12_default", "out", "case_elem_lik.txt"))
    for e, (r, row) in enumerate(zip(runs, rows)):
        want = tr["0_%d" % e]
        # the first iterations of M0, before FP32 rounding can move an MH decision
        np.testing.assert_allclose(r["trace"][0][:3], want[:3], rtol=1e-5, atol=1e-6)
        ref = [as_float(x) for x in row[2:5]]
        got = [r["loglik_null"], r["loglik_res"], r["loglik_all"]]
        assert np.all(np.abs(np.array(got) - ref) < 0.02 * np.abs(ref)), (got, ref)


def test_gbgc_chain_fp64_matches_oracle_st43(built):
    """43 taxa, elements of 150-700 columns with '-' as the gap character (so
    that taxa go missing and the outgroup path collapses), 30 + 90
    iterations: the device's traces and tables against the oracle's."""
    from oracle import pyoracle as po
    from phyloacc_gb300 import abi, synth
    ds = synth.make_dataset("st43", n_elements=6, seed=3)
    o = abi.gbgc_default_opts(ds.target)
    o.burnin, o.mcmc, o.seed, o.gapchar = 30, 90, 11, ord("-")
    runs = _ctx(ds, 0).gbgc_run(o, trace=True)
    for e, r in enumerate(runs):
        ref = po.gbgc_run(ds, o, e)
        assert r["status"] == ref["status"] == 0
        assert r["root"] == ref["root"]
        np.testing.assert_allclose(r["trace"], ref["trace"], rtol=1e-9, atol=1e-9, err_msg="element %d" % e)
        np.testing.assert_allclose([r["loglik_null"], r["loglik_res"], r["loglik_all"]],
                                   [ref["loglik_null"], ref["loglik_res"], ref["loglik_all"]], rtol=1e-9)
        np.testing.assert_allclose(r["max_loglik"], ref["max_loglik"], rtol=1e-9)
        np.testing.assert_allclose(r["rates"], ref["rates"], rtol=1e-9)
        np.testing.assert_allclose(r["post_b"], ref["post_b"], rtol=0, atol=1e-12)
        np.testing.assert_allclose(r["post_z"], ref["post_z"], rtol=0, atol=1e-12)
        assert (r["max_z"] == ref["max_z"]).all() and (r["max_b"] == ref["max_b"]).all()


def test_gbgc_chain_fp32_against_fp64_at_size(built):
    """120 taxa (the gBGC benchmark's tree and data), 48 elements, 100 + 400
    iterations: the FP32-partial chain against the FP64 one on the same
    elements and seed.  The chains part at the first MH decision that FP32
    rounding moves, so the marginal likelihoods are compared as two Monte
    Carlo estimates: within 1e-3 relative on every element and model, and
    1e-6 relative at the median (measured on GB300: 1.7e-4 and 4e-8)."""
    from phyloacc_gb300 import abi, synth
    ds = synth.make_dataset("gbgc120", n_elements=48, seed=5)
    o = abi.gbgc_default_opts(ds.target)
    o.burnin, o.mcmc, o.seed = 100, 400, 3
    r32 = _ctx(ds, 1).gbgc_run(o)
    r64 = _ctx(ds, 0).gbgc_run(o)
    rel = []
    for a, b in zip(r32, r64):
        assert a["status"] == b["status"]
        if a["status"] != 0:
            continue
        for k in ("loglik_null", "loglik_res", "loglik_all"):
            if np.isfinite(b[k]):
                rel.append(abs(a[k] - b[k]) / abs(b[k]))
    rel = np.array(rel)
    print("gbgc fp32 vs fp64: max %.3g median %.3g over %d" % (rel.max(), np.median(rel), len(rel)))
    assert len(rel) >= 100
    assert rel.max() < 1e-3 and np.median(rel) < 1e-6


@pytest.mark.parametrize("case", CASES + ["gbgc43_chain2"])
def test_gbgc_cli_matches_reference(built, tmp_path, case):
    """phyloacc-gbgc-gpu on the golden case's own cfg and inputs: every table
    the reference wrote (elem_lik, rate_postZ_{0,1,2}, 1_elem_Z,
    species_names) and every VERBOSE trace file."""
    import shutil
    import subprocess
    import phyloacc_gb300 as pg
    from golden_io import read_cfg
    src = os.path.join(GOLDEN, case)
    work = tmp_path / case
    shutil.copytree(src, work)
    shutil.rmtree(work / "out")
    os.makedirs(work / "out")
    r = subprocess.run([pg.CLI_GBGC_PATH, "case.cfg"], cwd=work, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    ref_dir = os.path.join(src, "out")
    for f in sorted(os.listdir(ref_dir)):
        lines1 = [ln.rstrip("\n").split("\t") for ln in open(os.path.join(ref_dir, f))]
        lines2 = [ln.rstrip("\n").split("\t") for ln in open(str(work / "out" / f))]
        assert len(lines1) == len(lines2), f
        assert lines1[0] == lines2[0], f
        for a, b in zip(lines1[1:], lines2[1:]):
            assert len(a) == len(b), f
            for x, y in zip(a, b):
                if x == y:
                    continue
                fx, fy = as_float(x), as_float(y)
                assert np.isclose(fx, fy, rtol=2e-6, atol=1e-12) or (np.isnan(fx) and np.isnan(fy)), (f, x, y)
    kv = read_cfg(str(work / "case.cfg"))
    T = int(kv["BURNIN"]) + int(kv["MCMC"])
    tr = np.load(os.path.join(src, "traces.npz"))
    chains = int(kv.get("CHAIN", 1))
    for key in tr.files:
        w = key.split("_")
        k = 1 if len(w) == 3 else 0                   # "m_e" or "m_e_c1"
        p = work / "out" / ("case_mcmc_trace_%s_%s.txt" % (w[0], w[1]))
        got = np.array([[float(v) for v in ln.rstrip("\n\t").split("\t")] for ln in list(open(p))[1:]])
        assert got.shape[0] == chains * T
        np.testing.assert_allclose(got[k * T:(k + 1) * T], tr[key], rtol=2e-7, atol=1e-300, err_msg=key)


def test_gbgc_served_equals_batch(built):
    """The serving form (pacc_gbgc_submit / poll / sync): every element
    served equals the same element run by pacc_gbgc_run, bit for bit, with
    the elements split over two submits, fewer slots than elements (eight),
    and a 0.1 ms idle bound between the submits (the blocks
    leave, the next submit launches again)."""
    import time
    from phyloacc_gb300 import abi, synth
    ds = synth.make_dataset("st43", n_elements=40, seed=9)
    o = abi.gbgc_default_opts(ds.target)
    o.burnin, o.mcmc, o.seed, o.gapchar = 20, 60, 5, ord("-")
    ref = {r["element_no"]: r for r in _ctx(ds, 1).gbgc_run(o)}
    from phyloacc_gb300 import Context
    so = abi.default_opts()
    so.precision = 1
    so.serve_idle_ns = 100000
    so.max_resident = 8
    ctx = Context(ds, so)
    ctx.gbgc_submit(o, elements=range(0, 25))
    got = []
    while len(got) < 25:
        got += ctx.gbgc_poll()
        time.sleep(0.01)
    time.sleep(0.05)                       # idle: the serving blocks leave
    ctx.gbgc_submit(o, elements=range(25, 40))
    ctx.gbgc_sync()
    got += ctx.gbgc_poll()
    assert sorted(r["element_no"] for r in got) == list(range(40))
    for r in got:
        w = ref[r["element_no"]]
        assert r["status"] == w["status"]
        if r["status"] != 0:
            continue
        for k in ("loglik_null", "loglik_res", "loglik_all"):
            assert r[k] == w[k] or (np.isnan(r[k]) and np.isnan(w[k])), (r["element_no"], k)
        assert (r["max_loglik"] == w["max_loglik"]).all() and (r["rates"] == w["rates"]).all()
        for k in ("max_z", "max_b", "post_b", "post_z"):
            assert (r[k] == w[k]).all(), (r["element_no"], k)


def test_gbgc_filtered_elements(built):
    """Elements the reference filters (more than CONSERVE_PROP of the
    conserved species missing, bpp_c.hpp:301-311) and elements whose tree
    collapses to a single taxon come back as PACC_FILTERED from both the
    batch and the serving paths, and the others are unaffected."""
    from phyloacc_gb300 import abi, synth
    ds = synth.make_dataset("st43", n_elements=6, seed=13)
    ds.bases = ds.bases.copy()
    S = ds.tree.n_species
    star = ord("*")
    blk = ds.element(1)
    for sp in ds.conserve:
        blk[sp, :] = star                     # every conserved species missing
    blk = ds.element(3)
    blk[:, :] = star
    blk[0, :] = ord("a")                      # one taxon left
    o = abi.gbgc_default_opts(ds.target)
    o.burnin, o.mcmc, o.seed = 10, 30, 2
    ref = _ctx(ds, 1).gbgc_run(o)
    assert [r["status"] for r in ref] == [0, 1, 0, 1, 0, 0]
    from phyloacc_gb300 import Context
    so = abi.default_opts()
    so.precision = 1
    ctx = Context(ds, so)
    ctx.gbgc_submit(o)
    ctx.gbgc_sync()
    got = {r["element_no"]: r for r in ctx.gbgc_poll()}
    assert sorted(got) == list(range(6))
    for e, r in enumerate(ref):
        assert got[e]["status"] == r["status"]
        if r["status"] == 0:
            assert got[e]["loglik_all"] == r["loglik_all"]


def test_gbgc_served_longer_element_recreates_slots(built):
    """A submit whose element is longer than the serving slots hold lets the
    running elements finish, re-creates the slots and goes on; every result
    equals the batch path's."""
    from phyloacc_gb300 import Context, abi, synth
    ds = synth.make_dataset("st43", n_elements=60, seed=21)
    short = [int(e) for e in np.flatnonzero(ds.lengths < 300)[:10]]
    long_ = [int(e) for e in np.flatnonzero(ds.lengths > 700)[:2]]
    assert len(short) == 10 and len(long_) == 2
    o = abi.gbgc_default_opts(ds.target)
    o.burnin, o.mcmc, o.seed, o.gapchar = 10, 30, 4, ord("-")
    ref = {r["element_no"]: r for r in _ctx(ds, 1).gbgc_run(o, elements=short + long_)}
    so = abi.default_opts()
    so.precision = 1
    ctx = Context(ds, so)
    ctx.gbgc_submit(o, elements=short)
    ctx.gbgc_submit(o, elements=long_)
    ctx.gbgc_sync()
    got = {r["element_no"]: r for r in ctx.gbgc_poll()}
    assert sorted(got) == sorted(short + long_)
    for e, r in got.items():
        assert r["loglik_all"] == ref[e]["loglik_all"] and (r["max_z"] == ref[e]["max_z"]).all()
