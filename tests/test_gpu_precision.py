"""FP32-partial precision path against FP64.

The FP32 path keeps partials in FP32 with exact power-of-two rescaling and
sums column log-likelihoods as an FP64 mantissa product with an integer
exponent; the eigensystem, exp(lambda r t), the chain's scalar arithmetic, the
MH ratio and the Z filter stay FP64.  Tolerances:
  * per-element log-likelihood: relative 1e-6 of the FP64 value;
  * chain summaries: FP32 vs FP64 under the same seed differ by no more than
    FP64 under two different seeds do (the Monte-Carlo error of the chain).
The underflow stress set (43 taxa, every branch x5, 2,000 bp columns, r2 = 6)
drives the partials through many rescales."""
import numpy as np
import pytest

import phyloacc_gb300 as pg
from oracle import pyoracle as po
from phyloacc_gb300 import abi, synth

pytestmark = pytest.mark.gpu

TOL_LL = 1e-6


def test_fp32_loglik_underflow_stress(built):
    ds = synth.make_dataset("st43_stress", n_elements=6, seed=3)
    o = abi.default_opts()
    o.precision = abi.PACC_FP32
    ctx = pg.Context(ds, o)
    rng = np.random.default_rng(4)
    for e in range(ds.n_elements):
        for _ in range(2):
            z = rng.integers(0, 3, ds.tree.n_nodes).astype(np.int32)
            rc, rn = rng.uniform(0.1, 0.9), 6.0
            a = ctx.loglik(e, z, rc, rn).sum()
            b = po.loglik(ds, o, e, z, rc, rn).sum()
            assert abs(a - b) <= TOL_LL * abs(b), (e, a, b)


@pytest.mark.parametrize("prec,cols", [(abi.PACC_FP32, 0), (abi.PACC_FP32_WARP, 1), (abi.PACC_FP32_WARP, 2),
                                       (abi.PACC_FP32_WARP, 4)])
def test_fp32_chain_tracks_fp64_on_stress_set(built, prec, cols):
    """While the FP32 and FP64 chains agree on Z and on every rate (the same
    draws and decisions; the CTA FP32 path draws its Gamma/Beta variates in
    FP32, so its rates agree to about 1e-7 relative), their log-likelihoods
    agree to 1e-6 relative; the chains may part later on a near-tie
    decision."""
    ds = synth.make_dataset("st43_stress", n_elements=4, seed=5)
    o = abi.default_opts()
    o.seed, o.burnin, o.mcmc, o.trace_iters = 2, 20, 40, 60
    o.precision = abi.PACC_FP64
    g64 = pg.Context(ds, o).run()
    o.precision = prec
    o.columns_per_lane = cols
    g32 = pg.Context(ds, o).run()
    compared = 0
    for e in range(ds.n_elements):
        for m in range(3):
            same = (g32.tr_z[e, m] == g64.tr_z[e, m]).all(axis=1)
            for k in ("n_rate", "c_rate", "g_rate", "l_rate"):
                same &= np.abs(g32.tr[k][e, m] - g64.tr[k][e, m]) <= 1e-5 * np.abs(g64.tr[k][e, m])
            upto = len(same) if same.all() else int(np.argmin(same))
            a, b = g32.tr["loglik"][e, m, :upto], g64.tr["loglik"][e, m, :upto]
            assert (np.abs(a - b) <= TOL_LL * np.abs(b)).all(), (e, m)
            compared += upto
    assert compared >= 60


def test_fp32_summaries_within_monte_carlo_error(built):
    ds = synth.make_dataset("st43", n_elements=24, seed=9)
    o = abi.default_opts()
    o.burnin, o.mcmc = 150, 450

    def run(prec, seed):
        o.precision, o.seed = prec, seed
        r = pg.Context(ds, o).run()
        ok = np.isin(r.status(), [abi.PACC_OK, abi.PACC_NAN_LIKELIHOOD])   # chains ran to the end
        ll = r.field("loglik")
        return ok, ll[:, 1] - ll[:, 0], r.post_z[:, 1, :, 3]

    ok0, bf_a, pacc_a = run(abi.PACC_FP64, 0)
    ok1, bf_b, pacc_b = run(abi.PACC_FP64, 1)
    ok2, bf_c, pacc_c = run(abi.PACC_FP32, 0)
    ok = ok0 & ok1 & ok2
    assert ok.sum() >= 16
    # posterior P(accelerated) of every branch under M1
    mc_p = np.mean(np.abs(pacc_b[ok] - pacc_a[ok]))
    assert np.mean(np.abs(pacc_c[ok] - pacc_a[ok])) <= 1.5 * mc_p + 1e-9
    # log Bayes factor M1 vs M0 where all three runs have a finite one (Eval2
    # gives -inf for degenerate configuration variances, as the reference does)
    fin = ok & np.isfinite(bf_a) & np.isfinite(bf_b) & np.isfinite(bf_c)
    if fin.sum() >= 3:
        mc_bf = np.mean(np.abs(bf_b[fin] - bf_a[fin]))
        assert np.mean(np.abs(bf_c[fin] - bf_a[fin])) <= 1.5 * mc_bf + 1e-9
