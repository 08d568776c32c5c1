"""pacc_pmatrix_noalloc: the P^T matrices of pacc_debug_pmatrix from a fixed
device scratch instead of per-call allocations (an entry point with no
counterpart in the reference).  Collected last, so it also runs after every
other test has used the device."""
import time

import numpy as np
import pytest

import phyloacc_gb300 as pg
from phyloacc_gb300 import abi, synth

pytestmark = pytest.mark.gpu

MAX_PAIRS = 4096   # PACC_NOALLOC_MAX_PAIRS in include/pacc.h


def test_noalloc_pmatrix_equals_allocating_entry_point_twice(built):
    ds = synth.make_dataset("st43", n_elements=2, seed=0)
    ctx = pg.Context(ds, abi.default_opts())
    rng = np.random.default_rng(11)
    for n in (257, MAX_PAIRS):          # two calls in a row, the second at the size limit
        d = np.concatenate([ds.tree.distances[:-1], rng.uniform(1e-6, 5.0, n)])[:n]
        r = rng.uniform(0.01, 8.0, n)
        d[:3] = [0.0, 1e-11, 1e-10]     # zero and near-zero branch lengths
        want = ctx.pmatrix(d, r)
        got = ctx.pmatrix_noalloc(d, r)
        assert np.array_equal(got, want)


def test_noalloc_pmatrix_refuses_oversize(built):
    ds = synth.make_dataset("st12", n_elements=2, seed=0)
    ctx = pg.Context(ds, abi.default_opts())
    with pytest.raises(pg.PaccError):
        ctx.pmatrix_noalloc(np.ones(MAX_PAIRS + 1), np.ones(MAX_PAIRS + 1))
    # the refusal leaves the entry point usable
    d, r = np.array([0.1, 0.2]), np.array([1.0, 2.0])
    assert np.array_equal(ctx.pmatrix_noalloc(d, r), ctx.pmatrix(d, r))


def test_noalloc_pmatrix_beside_a_serving_launch(built):
    """Called while a serving launch of the same context still has chains in
    flight, the entry point returns long before that launch drains (it runs on
    the context's second stream), and its matrices equal the allocating entry
    point's."""
    ds = synth.make_dataset("st43", n_elements=48, seed=14)
    o = abi.default_opts()
    o.seed, o.burnin, o.mcmc = 1, 500, 1500
    o.precision = abi.PACC_FP32
    o.sweeps_per_launch = 8
    o.block_threads, o.register_budget = 128, 128
    ctx = pg.Context(ds, o)
    d = np.concatenate([ds.tree.distances[:-1], [0.3, 1e-11, 0.0]])
    r = np.linspace(0.05, 6.0, len(d))
    first = ctx.pmatrix_noalloc(d, r)          # the set-up call, before the launch
    t0 = time.perf_counter()
    ctx.submit(ds, element_no=np.arange(ds.n_elements))
    ctx.poll(ds.n_elements)                    # the persistent launch is running
    t1 = time.perf_counter()
    got = ctx.pmatrix_noalloc(d, r)
    t_call = time.perf_counter() - t1
    in_flight = ctx.pending()
    while ctx.pending() > 0:
        ctx.poll(ds.n_elements)
    t_drain = time.perf_counter() - t0
    assert in_flight > 0, "the chains finished before the call returned"
    assert t_call < 0.25 * t_drain, (t_call, t_drain)
    want = ctx.pmatrix(d, r)
    assert np.array_equal(got, want)
    assert np.array_equal(first, want)
