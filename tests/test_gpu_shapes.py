"""Launch shapes of the CTA-per-chain kernel and its tuner.

Every alignment column is computed by one thread in the same arithmetic,
and the per-column log-likelihoods are summed exactly (64.64 fixed point),
so the threads per chain and the registers a thread (kernel instance) do
not change any result: the trial-launch tuner may pick any shape.  The
serving kernel's bounded wait for work (serve_idle_ns) ends idle blocks
without losing work."""
import numpy as np
import pytest

import phyloacc_gb300 as pg
from phyloacc_gb300 import abi, synth
from test_gpu_serving import _index, _same

pytestmark = pytest.mark.gpu


def _opts(prec, bt=0, regs=0):
    o = abi.default_opts()
    o.seed, o.burnin, o.mcmc, o.trace_iters = 3, 25, 55, 40
    o.precision = prec
    o.block_threads = bt
    o.register_budget = regs
    return o


@pytest.mark.parametrize("prec,shapes", [
    (abi.PACC_FP32, [(128, 128), (64, 128), (128, 168), (128, 255), (256, 255)]),
    (abi.PACC_FP64, [(128, 0), (64, 0), (256, 0)]),
])
def test_results_do_not_depend_on_launch_shape(built, prec, shapes):
    ds = synth.make_dataset("st43", n_elements=10, seed=11)
    runs = []
    for bt, regs in shapes:
        ctx = pg.Context(ds, _opts(prec, bt, regs))
        runs.append(ctx.run())
        sh = ctx.launch_shape()
        assert sh["block_threads"] == bt and sh["chains_per_sm"] >= 1
        if regs:
            assert sh["registers"] == regs
    ref = runs[0]
    for r in runs[1:]:
        for e in range(ds.n_elements):
            _same(r, e, ref, e)
        assert np.array_equal(r.tr["loglik"], ref.tr["loglik"])
        assert np.array_equal(r.tr_z, ref.tr_z)


def test_tuner_chooses_a_shape(built):
    ds = synth.make_dataset("st43", n_elements=200, seed=12)
    o = _opts(abi.PACC_FP32)
    o.burnin, o.mcmc, o.trace_iters = 6, 12, 0
    ctx = pg.Context(ds, o)
    r = ctx.run()
    assert (np.isin(r.status(), [abi.PACC_OK, abi.PACC_NAN_LIKELIHOOD, abi.PACC_FILTERED])).all()
    sh = ctx.launch_shape()
    assert sh["block_threads"] in (64, 128, 256)
    assert sh["registers"] in (128, 168, 255)
    assert sh["chains_per_sm"] >= 1
    assert sh["tuner_trial_ms"] >= 0
    # a fixed shape is taken as given
    o.block_threads, o.register_budget = 128, 168
    ctx2 = pg.Context(ds.subset(list(range(4))), o)
    ctx2.run()
    sh2 = ctx2.launch_shape()
    assert (sh2["block_threads"], sh2["registers"], sh2["tuner_trial_ms"]) == (128, 168, 0)


def test_serving_idle_bound_ends_idle_blocks_without_losing_work(built):
    """With a 0.1 ms bound the blocks that find no work leave at once (most
    blocks of a launch sized for the whole GPU get no element of a small
    batch); elements submitted later are taken by the blocks still running
    or by the next launch, and every result equals the batch run's."""
    ds = synth.make_dataset("st43", n_elements=24, seed=13)
    ref = pg.Context(ds, _opts(abi.PACC_FP32, 128, 128)).run()
    o = _opts(abi.PACC_FP32, 128, 128)
    o.sweeps_per_launch = 4
    o.serve_idle_ns = 100_000
    ctx = pg.Context(ds, o)
    got = []
    for ch in (list(range(0, 8)), list(range(8, 16)), list(range(16, 24))):
        ctx.submit(ds.subset(ch), element_no=np.asarray(ch))
        got.append(ctx.poll(24))
    while ctx.pending() > 0:
        got.append(ctx.poll(24))
    idx = _index(got)
    assert sorted(idx) == list(range(24))
    for e in range(24):
        r, i = idx[e]
        _same(r, i, ref, e)
    assert ctx.counters()["serve_idle_exits"] > 0
