"""The oracle against the reference's own outputs (tests/golden, written by
the unmodified PhyloAcc-ST sources built against the stand-in GSL/Armadillo
of oracle/shim and fed the same draw stream)."""
import numpy as np
import pytest

from golden_io import CASES, as_float, load_case, ref_tables, ref_traces
from oracle import pyoracle as po


def _check_tables(res, ds, tables, rel=6e-8, postz_only=False):
    if not postz_only:
        _check_lik_and_maxz(res, tables, rel)
    _check_postz(res, ds, tables)


def _check_lik_and_maxz(res, tables, rel):
    # _elem_lik.txt: precision 8
    _, rows = tables["elem_lik"]
    for i, row in enumerate(rows):
        assert int(row[0]) == i
        vals = [as_float(x) for x in row[2:]]
        m = res.field("loglik")[i]
        mx = res.field("max_loglik")[i]
        mine = [m[0], m[1], m[2], m[1] - m[0], m[1] - m[2], mx[0], mx[1], mx[2]]
        for a, b in zip(mine, vals):
            if np.isnan(b) or np.isinf(b):
                assert (np.isnan(a) and np.isnan(b)) or a == b
            else:
                assert abs(a - b) <= rel * max(1.0, abs(b)), (i, mine, vals)
    # _M*_elem_Z.txt: integers
    for m in range(3):
        _, rows = tables["M%d_elem_Z" % m]
        for i, row in enumerate(rows):
            assert [int(x) for x in row[1:]] == res.max_z[i, m].tolist()


def _check_postz(res, ds, tables):
    # _rate_postZ_M*.txt: default precision 6
    for m in range(3):
        _, rows = tables["rate_postZ_M%d" % m]
        st = res.status()
        k = 0
        for i in range(ds.n_elements):
            if st[i] == 1:
                continue
            row = [as_float(x) for x in rows[k]]
            k += 1
            assert int(row[0]) == i
            f = res.arr[i].model[m]
            mine = [f.n_rate, f.c_rate, f.g_rate, f.l_rate, f.l2_rate] + res.post_z[i, m].reshape(-1).tolist()
            assert np.allclose(mine, row[1:], rtol=6e-6, atol=1e-12), (i, m)


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference(case):
    ds, o, kv = load_case(case)
    o.trace_iters = 200
    res = po.run(ds, o, threads=4)
    _check_tables(res, ds, ref_tables(case))
    tr = ref_traces(case)
    N = ds.tree.n_nodes
    for key, a in tr.items():
        m, e = int(key[1]), int(key.split("_")[1])
        T = a.shape[0]
        mine = np.stack([res.tr[k][e, m, :T] for k in ("loglik", "n_rate", "c_rate", "g_rate", "l_rate", "l2_rate")], 1)
        assert np.allclose(mine, a[:, :6], rtol=6e-8, atol=1e-300), (case, key)
        assert (res.tr_z[e, m, :T] == a[:, 6:6 + N].astype(np.int8)).all(), (case, key)


def test_oracle_matches_reference_continued_chain():
    """CHAIN 2: the reference runs every element again from SEED, starting
    from Z = 0 on every node; it appends the second chain's _rate_postZ rows
    and trace rows and rewrites _elem_lik / _elem_Z with the second chain's."""
    case = "st12_chain2"
    ds, o, kv = load_case(case)
    assert kv["CHAIN"] == "2"
    o.trace_iters = 200
    res = [po.run(ds, o, threads=4, chain=k) for k in range(2)]
    tables = ref_tables(case)
    n = int(sum(res[0].status() != 1))
    for k in range(2):
        part = dict(tables)
        for m in range(3):
            hdr, rows = tables["rate_postZ_M%d" % m]
            assert len(rows) == 2 * n
            part["rate_postZ_M%d" % m] = (hdr, rows[k * n:(k + 1) * n])
        _check_tables(res[k], ds, part, postz_only=(k == 0))
    N = ds.tree.n_nodes
    tr = ref_traces(case)
    assert any(key.endswith("_c1") for key in tr)
    for key, a in tr.items():
        k = 1 if key.endswith("_c1") else 0
        m, e = int(key[1]), int(key.split("_")[1])
        r = res[k]
        T = a.shape[0]
        mine = np.stack([r.tr[f][e, m, :T] for f in ("loglik", "n_rate", "c_rate", "g_rate", "l_rate", "l2_rate")], 1)
        assert np.allclose(mine, a[:, :6], rtol=6e-8, atol=1e-300), (case, key)
        assert (r.tr_z[e, m, :T] == a[:, 6:6 + N].astype(np.int8)).all(), (case, key)
    # the second chain really starts elsewhere: Z = 0 on every node at iteration 0
    assert (res[1].tr_z[:, :, 0] == 0).all()


def test_oracle_matches_reference_sample_hyper():
    """SAMPLE_HYPER with CHAIN 3: only M2 runs, each chain from the state the
    previous one left, and the hyper-parameters are drawn between chains.
    The reference appends per chain a _hyper.txt row, an _elem_lik.txt row
    per element (No, ID, loglik_all, loglik_Max) and the _rate_postZ_M2 rows."""
    case = "st12_hyper"
    ds, o, kv = load_case(case)
    assert kv["SAMPLE_HYPER"] == "1"
    K, n, N = int(kv["CHAIN"]), ds.n_elements, ds.tree.n_nodes
    o.trace_iters = 200
    res, hyper = po.run_hyper(ds, o, K, threads=4)
    tables = ref_tables(case)
    _, rows = tables["hyper"]
    assert len(rows) == K + 1
    assert np.allclose([as_float(x) for x in rows[0][1:]], hyper[0, :8])
    for k in range(K):
        row = [as_float(x) for x in rows[k + 1]]
        assert int(row[0]) == k
        assert np.allclose(row[1:], hyper[k + 1], rtol=6e-6, atol=0), (k, row, hyper[k + 1])
    assert not np.allclose(hyper[K], hyper[0])          # some proposals were accepted
    _, rows = tables["elem_lik"]
    assert len(rows) == K * n
    st = res.status()
    for k in range(K):
        for i in range(n):
            row = rows[k * n + i]
            r = res.arr[k * n + i]
            assert int(row[0]) == i
            for a, b in zip([r.model[2].loglik, r.model[2].max_loglik], [as_float(x) for x in row[2:]]):
                if st[k * n + i] == 1:
                    assert b == 0                           # filtered: the slot's initial zero
                elif np.isinf(b) or np.isnan(b):
                    assert a == b or (np.isnan(a) and np.isnan(b))
                else:
                    assert abs(a - b) <= 6e-8 * max(1.0, abs(b)), (k, i, a, b)
    for m in (0, 1):
        assert tables["rate_postZ_M%d" % m][1] == []
    _, rows = tables["rate_postZ_M2"]
    kept = [j for j in range(K * n) if st[j] != 1]
    assert len(rows) == len(kept)
    for row, j in zip(rows, kept):
        row = [as_float(x) for x in row]
        f = res.arr[j].model[2]
        mine = [f.n_rate, f.c_rate, f.g_rate, f.l_rate, f.l2_rate] + res.post_z[j, 2].reshape(-1).tolist()
        assert int(row[0]) == j % n
        assert np.allclose(mine, row[1:], rtol=6e-6, atol=1e-12), j
    for key, a in ref_traces(case).items():
        w = key.split("_")
        k = int(w[2][1:]) if len(w) == 3 else 0
        j = k * n + int(w[1])
        T = a.shape[0]
        mine = np.stack([res.tr[f][j, 2, :T] for f in ("loglik", "n_rate", "c_rate", "g_rate", "l_rate", "l2_rate")], 1)
        assert np.allclose(mine, a[:, :6], rtol=6e-8, atol=1e-300), key
        assert (res.tr_z[j, 2, :T] == a[:, 6:6 + N].astype(np.int8)).all(), key


def test_gbgc_fixture_layout():
    """The gBGC fixture (src/PhyloAcc-ST-GBGC run on the 12-taxon inputs):
    per-iteration traces (loglik, rate_n, rate_c, GB, then B and Z of every
    node) and per-element tables, kept for the gBGC oracle and kernels."""
    ds, o, kv = load_case("gbgc12_default")
    N, n = ds.tree.n_nodes, ds.n_elements
    T = int(kv["BURNIN"]) + int(kv["MCMC"])
    tr = ref_traces("gbgc12_default")
    assert sorted(tr) == sorted("%d_%d" % (m, e) for m in range(3) for e in range(n))
    for a in tr.values():
        assert a.shape == (T, 4 + 2 * N)
        assert np.isfinite(a[:, 0]).all()
        assert set(np.unique(a[:, 4 + N:])) <= {-1, 0, 1, 2}
    tables = ref_tables("gbgc12_default")
    hdr, rows = tables["elem_lik"]
    assert hdr[:3] == ["No.", "ID", "loglik_NUll"] and len(rows) == n
    hdr, rows = tables["1_elem_Z"]
    assert len(rows) == n and hdr[0] == ds.tree.names[0] + "_B"
