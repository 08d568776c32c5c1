"""GPU parity: every kernel of the chain against the oracle on the same
inputs and draw stream, and the whole path against the reference's own
outputs (tests/golden)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import phyloacc_gb300 as pg
from golden_io import CASES, as_float, load_case, read_cfg, read_table, ref_tables, ref_traces
from oracle import pyoracle as po
from phyloacc_gb300 import abi, synth
from test_oracle_golden import _check_tables

pytestmark = pytest.mark.gpu


def test_stream_words_match_oracle(built):
    for seed, w0 in [(0, 0), (5, 12345), (7, 2**33 + 3)]:
        assert (pg.stream_words(seed, w0, 4099) == po.stream(seed, w0, 4099)).all()


def test_pmatrix_matches_oracle(built):
    ds = synth.make_dataset("st43", n_elements=2, seed=0)
    o = abi.default_opts()
    ctx = pg.Context(ds, o)
    rng = np.random.default_rng(0)
    d = np.concatenate([ds.tree.distances[:-1], rng.uniform(1e-6, 5.0, 200)])
    r = np.concatenate([np.full(ds.tree.n_nodes - 1, 0.35), rng.uniform(0.01, 8.0, 200)])
    a = ctx.pmatrix(d, r)
    b = po.pmatrix(ds, o, d, r)
    assert np.abs(a - b).max() < 1e-14 * 4
    assert np.abs(a.sum(1) - 1).max() < 1e-13      # P^T columns are distributions over the child base


@pytest.mark.parametrize("prec,tol", [(abi.PACC_FP64, 1e-12), (abi.PACC_FP32, 1e-6)])
def test_loglik_matches_oracle(built, prec, tol):
    for kind, elems in [("st12", [0, 1, 90, 95]), ("st43", [0, 3, 17])]:
        ds = synth.make_dataset(kind, n_elements=100, seed=1)
        o = abi.default_opts()
        o.precision = prec
        ctx = pg.Context(ds, o)
        rng = np.random.default_rng(2)
        for e in elems:
            for _ in range(3):
                z = rng.integers(0, 3, ds.tree.n_nodes).astype(np.int32)
                rc, rn = rng.uniform(0.1, 0.9), rng.uniform(1.0, 6.0)
                a = ctx.loglik(e, z, rc, rn)
                b = po.loglik(ds, o, e, z, rc, rn)
                assert abs(a.sum() - b.sum()) <= tol * abs(b.sum()), (kind, e, a.sum(), b.sum())
                assert (np.abs(a - b) <= tol * np.maximum(1.0, np.abs(b)) * (10 if prec else 1)).all()


def _chain_compare(ds, o, T=200):
    o.trace_iters = T
    g = pg.Context(ds, o).run()
    r = po.run(ds, o, threads=0)
    assert (g.status() == r.status()).all()
    for e in range(ds.n_elements):
        if r.status()[e] == abi.PACC_FILTERED:
            continue
        for m in range(3):
            assert (g.tr_z[e, m] == r.tr_z[e, m]).all(), (e, m)
            ll_g, ll_r = g.tr["loglik"][e, m], r.tr["loglik"][e, m]
            assert (np.abs(ll_g - ll_r) <= 1e-12 * np.abs(ll_r)).all(), (e, m)
            for k in ("n_rate", "c_rate", "g_rate", "l_rate", "l2_rate"):
                a, b = g.tr[k][e, m], r.tr[k][e, m]
                assert (np.abs(a - b) <= 1e-12 * np.abs(b) + 1e-300).all(), (e, m, k)
    return g, r


def test_chain_matches_oracle_first_200_iterations(built):
    ds = synth.make_dataset("st12", seed=0).subset([0, 1, 2, 3, 80, 90, 91, 99])
    o = abi.default_opts()
    o.seed, o.burnin, o.mcmc = 0, 100, 300
    g, r = _chain_compare(ds, o)
    mg, mr = g.field("loglik"), r.field("loglik")
    fin = np.isfinite(mr)
    assert np.allclose(mg[fin], mr[fin], rtol=1e-10, atol=0)
    assert (g.max_z == r.max_z).all()
    assert np.abs(g.post_z - r.post_z).max() == 0


def test_chain_matches_oracle_43_taxa(built):
    ds = synth.make_dataset("st43", n_elements=60, seed=0).subset([0, 5, 11, 23])
    o = abi.default_opts()
    o.seed, o.burnin, o.mcmc = 3, 60, 140
    _chain_compare(ds, o)


@pytest.mark.parametrize("case", CASES)
def test_gpu_matches_reference_golden(built, case):
    ds, o, kv = load_case(case)
    o.trace_iters = 200
    res = pg.Context(ds, o).run()
    _check_tables(res, ds, ref_tables(case))
    tr = ref_traces(case)
    N = ds.tree.n_nodes
    for key, a in tr.items():
        m, e = int(key[1]), int(key.split("_")[1])
        T = a.shape[0]
        mine = np.stack([res.tr[k][e, m, :T] for k in ("loglik", "n_rate", "c_rate", "g_rate", "l_rate", "l2_rate")], 1)
        assert np.allclose(mine, a[:, :6], rtol=6e-8, atol=1e-300), (case, key)
        assert (res.tr_z[e, m, :T] == a[:, 6:6 + N].astype(np.int8)).all(), (case, key)


@pytest.mark.parametrize("case", CASES)
def test_cli_drop_in_matches_reference_tables(built, case, tmp_path):
    src = os.path.join(os.path.dirname(__file__), "golden", case)
    work = tmp_path / case
    shutil.copytree(src, work)
    shutil.rmtree(work / "out")
    os.makedirs(work / "out")
    r = subprocess.run([pg.CLI_PATH, "case.cfg"], cwd=work, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    ref_dir = os.path.join(src, "out")
    for f in sorted(os.listdir(ref_dir)):
        h1, rows1 = read_table(os.path.join(ref_dir, f))
        h2, rows2 = read_table(str(work / "out" / f))
        assert h1 == h2, f
        assert len(rows1) == len(rows2), f
        for a, b in zip(rows1, rows2):
            assert len(a) == len(b), f
            for x, y in zip(a, b):
                if x == y:
                    continue
                fx, fy = as_float(x), as_float(y)
                assert np.isclose(fx, fy, rtol=2e-7, atol=1e-12) or (np.isnan(fx) and np.isnan(fy)), (f, x, y)
    # VERBOSE traces
    for key, a in ref_traces(case).items():
        m, e = key.split("_")
        p = work / "out" / ("case_mcmc_trace_%s_%s.txt" % (m, e))
        got = np.array([[float(v) for v in ln.rstrip("\n\t").split("\t")] for ln in list(open(p))[1:]])
        assert np.allclose(got[:a.shape[0]], a, rtol=2e-7, atol=1e-300), key


def test_later_chain_matches_oracle(built):
    """A later chain of a CHAIN > 1 run (every element again from SEED,
    starting from Z = 0 on every node) reproduces the oracle's chains."""
    ds, o, kv = load_case("st12_chain2")
    o.trace_iters = 200
    o.chain = 1
    g = pg.Context(ds, o).run()
    r = po.run(ds, o, threads=4, chain=1)
    assert (g.tr_z[:, :, 0] == 0).all()
    assert (g.tr_z == r.tr_z).all()
    rel = np.abs(g.tr["loglik"] - r.tr["loglik"]) / np.abs(r.tr["loglik"])
    assert rel.max() < 1e-12
    mg, mr = g.field("loglik"), r.field("loglik")
    assert (np.isclose(mg, mr, rtol=1e-10, atol=0) | (np.isinf(mg) & np.isinf(mr))).all()
    assert (g.max_z == r.max_z).all()


def test_cli_two_chains_match_reference(built, tmp_path):
    """CHAIN 2 through phyloacc-st-gpu: the reference's tables (the second
    chain's _elem_lik and _elem_Z, both chains' _rate_postZ rows) and both
    chains' trace rows."""
    case = "st12_chain2"
    src = os.path.join(os.path.dirname(__file__), "golden", case)
    work = tmp_path / case
    shutil.copytree(src, work)
    shutil.rmtree(work / "out")
    os.makedirs(work / "out")
    r = subprocess.run([pg.CLI_PATH, "case.cfg"], cwd=work, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    ref_dir = os.path.join(src, "out")
    for f in sorted(os.listdir(ref_dir)):
        h1, rows1 = read_table(os.path.join(ref_dir, f))
        h2, rows2 = read_table(str(work / "out" / f))
        assert h1 == h2, f
        assert len(rows1) == len(rows2), f
        for a, b in zip(rows1, rows2):
            assert len(a) == len(b), f
            for x, y in zip(a, b):
                if x == y:
                    continue
                fx, fy = as_float(x), as_float(y)
                assert np.isclose(fx, fy, rtol=2e-7, atol=1e-12) or (np.isnan(fx) and np.isnan(fy)), (f, x, y)
    kv = read_cfg(str(work / "case.cfg"))
    T = int(kv["BURNIN"]) + int(kv["MCMC"])
    for key, a in ref_traces(case).items():
        w = key.split("_")
        k = 1 if len(w) == 3 else 0
        p = work / "out" / ("case_mcmc_trace_%s_%s.txt" % (w[0], w[1]))
        got = np.array([[float(v) for v in ln.rstrip("\n\t").split("\t")] for ln in list(open(p))[1:]])
        assert got.shape[0] == 2 * T
        assert np.allclose(got[k * T:k * T + a.shape[0]], a, rtol=2e-7, atol=1e-300), key


def test_sample_hyper_chains_match_oracle(built):
    """SAMPLE_HYPER chains through the API: M2 only, each chain from the end
    state the previous one returned, with the priors the oracle's
    hyper-parameter MH drew; traces, marginal likelihoods and end states equal
    the oracle's."""
    ds, o, kv = load_case("st12_hyper")
    K, n, N = int(kv["CHAIN"]), ds.n_elements, ds.tree.n_nodes
    o.trace_iters = 200
    ref, hyper = po.run_hyper(ds, o, K, threads=4)
    o.sample_hyper = 1
    start_z, start_rates = None, None
    for k in range(K):
        ok = o
        (ok.acce_prior_a, ok.acce_prior_b, ok.conserve_prior_a, ok.conserve_prior_b, ok.hyper_lrate_a,
         ok.hyper_lrate_b, ok.hyper_grate_a, ok.hyper_grate_b, ok.hyper_lrate2_a, ok.hyper_lrate2_b) = hyper[k]
        g = pg.Context(ds, ok).run(start_z=start_z, start_rates=start_rates)
        for i in range(n):
            j = k * n + i
            assert (g.tr_z[i, 2] == ref.tr_z[j, 2]).all(), (k, i)
            rel = np.abs(g.tr["loglik"][i, 2] - ref.tr["loglik"][j, 2]) / np.abs(ref.tr["loglik"][j, 2])
            assert rel.max() < 1e-12, (k, i)
            a, b = g.arr[i].model[2].loglik, ref.arr[j].model[2].loglik
            assert np.isclose(a, b, rtol=1e-10, atol=0) or (np.isinf(a) and a == b), (k, i, a, b)
            assert (g.end_z[i] == ref.end_z[j]).all(), (k, i)
            assert np.allclose(list(g.arr[i].end_rates), list(ref.arr[j].end_rates), rtol=1e-12, atol=0), (k, i)
            assert g.arr[i].model[0].loglik == 0 and g.arr[i].model[1].loglik == 0
        start_z = g.end_z[:n].copy()
        start_rates = np.array([list(g.arr[i].end_rates) for i in range(n)])


def _cli_tables_match(src, work):
    ref_dir = os.path.join(src, "out")
    for f in sorted(os.listdir(ref_dir)):
        h1, rows1 = read_table(os.path.join(ref_dir, f))
        h2, rows2 = read_table(str(work / "out" / f))
        assert h1 == h2, f
        assert len(rows1) == len(rows2), f
        for a, b in zip(rows1, rows2):
            assert len(a) == len(b), f
            for x, y in zip(a, b):
                if x == y:
                    continue
                fx, fy = as_float(x), as_float(y)
                assert np.isclose(fx, fy, rtol=2e-7, atol=1e-12) or (np.isnan(fx) and np.isnan(fy)), (f, x, y)


def test_cli_sample_hyper_matches_reference(built, tmp_path):
    """SAMPLE_HYPER with CHAIN 3 through phyloacc-st-gpu: the reference's
    _hyper.txt rows, per-chain _elem_lik.txt and _rate_postZ_M2.txt rows, and
    every chain's M2 trace."""
    case = "st12_hyper"
    src = os.path.join(os.path.dirname(__file__), "golden", case)
    work = tmp_path / case
    shutil.copytree(src, work)
    shutil.rmtree(work / "out")
    os.makedirs(work / "out")
    r = subprocess.run([pg.CLI_PATH, "case.cfg"], cwd=work, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    _cli_tables_match(src, work)
    kv = read_cfg(str(work / "case.cfg"))
    T, K = int(kv["BURNIN"]) + int(kv["MCMC"]), int(kv["CHAIN"])
    for key, a in ref_traces(case).items():
        w = key.split("_")
        k = int(w[2][1:]) if len(w) == 3 else 0
        p = work / "out" / ("case_mcmc_trace_%s_%s.txt" % (w[0], w[1]))
        got = np.array([[float(v) for v in ln.rstrip("\n\t").split("\t")] for ln in list(open(p))[1:]])
        assert got.shape[0] == K * T
        assert np.allclose(got[k * T:k * T + a.shape[0]], a, rtol=2e-7, atol=1e-300), key


@pytest.mark.parametrize("cols", [1, 2])
def test_batched_layout_fp64_matches_oracle(built, cols):
    """The warp-per-chain layout with FP64 partials reproduces the oracle's
    chains, with one or two alignment columns per lane."""
    ds = synth.make_dataset("st12", seed=0).subset([0, 1, 2, 3, 80, 90, 91, 99])
    o = abi.default_opts()
    o.seed, o.burnin, o.mcmc = 0, 100, 300
    o.precision = abi.PACC_FP64_BATCHED
    o.columns_per_lane = cols
    g, r = _chain_compare(ds, o)
    mg, mr = g.field("loglik"), r.field("loglik")
    fin = np.isfinite(mr)
    assert np.allclose(mg[fin], mr[fin], rtol=1e-10, atol=0)
    assert (g.max_z == r.max_z).all()


def test_batched_layout_fp64_43_taxa_resumable(built):
    """Chains advanced a few iterations per launch equal chains run in one launch."""
    ds = synth.make_dataset("st43", n_elements=60, seed=0).subset([0, 5, 11, 23, 40])
    o = abi.default_opts()
    o.seed, o.burnin, o.mcmc = 3, 60, 140
    o.precision = abi.PACC_FP64_BATCHED
    g1, r = _chain_compare(ds, o)
    o.sweeps_per_launch = 7
    g2 = pg.Context(ds, o).run()
    assert (g2.tr_z == g1.tr_z).all()
    assert np.array_equal(g2.field("loglik"), g1.field("loglik"))


def test_contexts_with_different_models_interleave(built):
    """Each context launches with its own tree and rate matrix, whatever
    context ran last on the device."""
    a = synth.make_dataset("st12", seed=0).subset([0, 1, 2])
    b = synth.make_dataset("st43", n_elements=3, seed=1)
    o = abi.default_opts()
    o.seed, o.burnin, o.mcmc = 1, 20, 40
    ca, cb = pg.Context(a, o), pg.Context(b, o)
    r1 = ca.run()
    cb.run()
    r2 = ca.run()
    assert np.array_equal(r1.field("loglik"), r2.field("loglik"))
    assert np.array_equal(r1.post_z, r2.post_z)
    assert np.allclose(ca.pmatrix(a.tree.distances[:4], np.ones(4)), po.pmatrix(a, o, a.tree.distances[:4], np.ones(4)),
                       rtol=0, atol=1e-14)
