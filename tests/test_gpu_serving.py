"""Serving mode (continuous batching).  CTA-per-chain layout: a persistent
kernel takes element slots from a queue the host appends to while it runs.
Warp-per-chain layout: chains stay resident in device slots, are advanced by
sweep steps, queued elements are admitted as slots free up and finished
chains are retired after every step.  An element's chain depends only on the element, the model and SEED
(every element restarts the same draw stream), so a served element must give
bit-identical results to the same element run in a batch, whatever else is
resident beside it and whenever it was admitted."""
import numpy as np
import pytest

import phyloacc_gb300 as pg
from phyloacc_gb300 import abi, synth

pytestmark = pytest.mark.gpu

FIELDS = ("loglik", "max_loglik", "n_rate", "c_rate", "g_rate", "l_rate", "l2_rate", "failure", "n_configs")


def _opts(prec, sweeps=0, max_resident=0, trace=0):
    o = abi.default_opts()
    o.seed, o.burnin, o.mcmc = 4, 30, 70
    o.precision = prec
    o.sweeps_per_launch = sweeps
    o.max_resident = max_resident
    o.trace_iters = trace
    return o


def _index(results):
    """element_no -> (Results, row) over several poll() results."""
    out = {}
    for r in results:
        for i in range(r.n):
            no = int(r.arr[i].element_no)
            assert no not in out, "element %d returned twice" % no
            out[no] = (r, i)
    return out


def _same(a, ia, b, ib):
    assert a.arr[ia].status == b.arr[ib].status
    for m in range(3):
        for f in FIELDS:
            x, y = getattr(a.arr[ia].model[m], f), getattr(b.arr[ib].model[m], f)
            assert x == y or (np.isnan(x) and np.isnan(y)), (m, f, x, y)
    assert (a.max_z[ia] == b.max_z[ib]).all()
    assert np.array_equal(a.post_z[ia], b.post_z[ib])


def _serve(ds, o, chunks, polls_between=2):
    ctx = pg.Context(ds, o)
    got = []
    for ch in chunks:
        ctx.submit(ds.subset(ch), element_no=np.asarray(ch))
        for _ in range(polls_between):
            got.append(ctx.poll(len(ds.lengths)))
    while ctx.pending() > 0:
        got.append(ctx.poll(len(ds.lengths)))
    return _index(got)


ALL = [abi.PACC_FP32, abi.PACC_FP64, abi.PACC_FP32_WARP, abi.PACC_FP64_BATCHED]


@pytest.mark.parametrize("prec", ALL)
def test_served_equals_batched(built, prec):
    ds = synth.make_dataset("st43", n_elements=30, seed=5)
    ref = pg.Context(ds, _opts(prec)).run()
    chunks = [list(range(0, 9)), list(range(9, 21)), list(range(21, 30))]
    got = _serve(ds, _opts(prec, sweeps=3, max_resident=7), chunks)
    assert sorted(got) == list(range(30))
    for e in range(30):
        r, i = got[e]
        _same(r, i, ref, e)
        if r.arr[i].status == abi.PACC_OK:
            assert r.arr[i].latency_ms > 0


@pytest.mark.parametrize("prec", [abi.PACC_FP32, abi.PACC_FP32_WARP])
def test_alone_equals_mixed(built, prec):
    ds = synth.make_dataset("st43", n_elements=40, seed=6)
    x = 17
    alone = _serve(ds, _opts(prec, sweeps=5), [[x]])
    mixed = _serve(ds, _opts(prec, sweeps=5, max_resident=12),
                   [list(range(0, 10)), [x] + list(range(20, 40)), list(range(10, 17))])
    a, ia = alone[x]
    b, ib = mixed[x]
    _same(a, ia, b, ib)


@pytest.mark.parametrize("prec", [abi.PACC_FP32, abi.PACC_FP32_WARP])
def test_memory_budget_too_small_is_refused(built, prec):
    ds = synth.make_dataset("st43", n_elements=4, seed=7)
    o = _opts(prec, sweeps=3)
    o.memory_budget_bytes = 1 << 20
    ctx = pg.Context(ds, o)
    with pytest.raises(pg.PaccError):
        ctx.submit(ds)


@pytest.mark.parametrize("prec", [abi.PACC_FP32, abi.PACC_FP32_WARP])
def test_served_filtered_elements_return_at_once(built, prec):
    ds = synth.make_dataset("st43", n_elements=12, seed=8)
    o = _opts(prec, sweeps=4)
    o.min_len = 10**6          # every element is filtered before it reaches a slot
    ctx = pg.Context(ds, o)
    ctx.submit(ds)
    r = ctx.poll(12)
    assert r.n == 12
    assert (r.status()[:12] == abi.PACC_FILTERED).all()
    assert ctx.pending() == 0


def test_longer_element_recreates_serving_slots(built):
    """CTA serving sizes its slots for 5,120 columns at the first submit; a
    later element of 6,000 columns lets the running chains finish, the slots
    are made again, and every element still equals its batched run."""
    import dataclasses
    ds = synth.make_dataset("st43", n_elements=60, seed=5)
    S = ds.tree.n_species
    long_cols = np.concatenate([ds.element(e) for e in range(20, 60)], axis=1)[:, :6000]
    assert long_cols.shape[1] == 6000
    blocks = [ds.element(e) for e in range(8)] + [long_cols, np.ascontiguousarray(long_cols[:, ::-1])]
    lens = np.array([b.shape[1] for b in blocks], np.int32)
    offs = np.zeros(len(blocks), np.int64)
    offs[1:] = np.cumsum(lens[:-1].astype(np.int64) * S)
    mix = dataclasses.replace(ds, lengths=lens, offsets=offs, bases=np.concatenate([b.reshape(-1) for b in blocks]),
                              element_names=["e%d" % i for i in range(10)], accelerated=np.zeros(10, bool),
                              r1=np.zeros(10), r2=np.zeros(10))
    ctx = pg.Context(mix, _opts(abi.PACC_FP32, sweeps=3))
    ctx.submit(mix.subset(list(range(8))), element_no=np.arange(8))
    got = [ctx.poll(10)]
    ctx.submit(mix.subset([8, 9]), element_no=np.array([8, 9]))
    while ctx.pending() > 0:
        got.append(ctx.poll(10))
    got = _index(got)
    assert sorted(got) == list(range(10))
    ref = pg.Context(mix, _opts(abi.PACC_FP32)).run()
    for e in range(10):
        r, i = got[e]
        assert r.arr[i].status == abi.PACC_OK
        _same(r, i, ref, e)
    assert ctx.counters()["kernel_ms"] > 0
