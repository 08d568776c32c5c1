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


def _pacc_batch_se(tr_z, burn, n_batches=20):
    """Batch-means Monte-Carlo standard error of P(Z = 2) per node from a
    chain's Z trace [T][N] (post-burn-in samples split into n_batches)."""
    x = (tr_z[burn:] == 2).astype(np.float64)
    b = x.shape[0] // n_batches
    means = x[:n_batches * b].reshape(n_batches, b, -1).mean(axis=1)
    return means.std(axis=0, ddof=1) / np.sqrt(n_batches)


def _within(pa, sa, pb, sb, mcmc, z=4.0):
    """Fraction of posteriors whose difference lies within z combined
    batch-means standard errors (plus one sample's weight)."""
    return float(np.mean(np.abs(pa - pb) <= z * np.sqrt(sa ** 2 + sb ** 2) + 1.0 / mcmc))


def test_fp32_summaries_within_monte_carlo_error(built):
    """64 elements of the 43-taxon workload at the benchmarked chain length
    (BURNIN 500 + MCMC 1500), FP32 against FP64 under the same seed:
      * P(accelerated) of every branch under M1 and M2: the difference lies
        within four batch-means standard errors of the two chains for as many
        branches as it does between two FP64 chains with different seeds;
      * both log Bayes factors, logBF1 = M1 - M0 and logBF2 = M1 - M2: the
        FP32 - FP64 differences are no larger than the FP64 seed-to-seed
        differences (median and mean over elements, 1.5x allowance)."""
    ds = synth.make_dataset("st43", n_elements=64, seed=9)
    o = abi.default_opts()
    o.burnin, o.mcmc, o.trace_iters = 500, 1500, 2000

    def run(prec, seed):
        o.precision, o.seed = prec, seed
        r = pg.Context(ds, o).run()
        ok = np.isin(r.status(), [abi.PACC_OK, abi.PACC_NAN_LIKELIHOOD])   # chains ran to the end
        ll = r.field("loglik")
        se = np.array([[_pacc_batch_se(r.tr_z[e, m], o.burnin) for m in (1, 2)] for e in range(ds.n_elements)])
        return ok, ll[:, 1] - ll[:, 0], ll[:, 1] - ll[:, 2], r.post_z[:, 1:, :, 3], se

    ok0, bf1_a, bf2_a, p_a, se_a = run(abi.PACC_FP64, 0)
    ok1, bf1_b, bf2_b, p_b, se_b = run(abi.PACC_FP64, 1)
    ok2, bf1_c, bf2_c, p_c, se_c = run(abi.PACC_FP32, 0)
    ok = ok0 & ok1 & ok2
    assert ok.sum() >= 48
    # P(accelerated) per branch, M1 and M2
    f32 = _within(p_c[ok], se_c[ok], p_a[ok], se_a[ok], o.mcmc)
    f64 = _within(p_b[ok], se_b[ok], p_a[ok], se_a[ok], o.mcmc)
    assert f32 >= 0.95 and f32 >= f64 - 0.02, (f32, f64)
    # both log Bayes factors where all three runs have finite ones (Eval2
    # gives -inf for degenerate configuration variances, as the reference does)
    for a, b, c in ((bf1_a, bf1_b, bf1_c), (bf2_a, bf2_b, bf2_c)):
        fin = ok & np.isfinite(a) & np.isfinite(b) & np.isfinite(c)
        assert fin.sum() >= 16
        d32, d64 = np.abs(c[fin] - a[fin]), np.abs(b[fin] - a[fin])
        assert np.median(d32) <= 1.5 * np.median(d64) + 1e-9, (np.median(d32), np.median(d64))
        assert np.mean(d32) <= 1.5 * np.mean(d64) + 1e-9, (np.mean(d32), np.mean(d64))


def test_fp32_loglik_stress_set_at_size(built):
    """The underflow stress set at its stated size: 1,000 elements of
    2,000 bp on the 43-taxon tree with every branch x5 and r2 = 6.  Per
    element, the FP32 likelihood kernel against the FP64 one at a random
    state: relative error <= 1e-6."""
    ds = synth.make_dataset("st43_stress", n_elements=1000, seed=3)
    o = abi.default_opts()
    o.precision = abi.PACC_FP32
    c32 = pg.Context(ds, o)
    o.precision = abi.PACC_FP64
    c64 = pg.Context(ds, o)
    rng = np.random.default_rng(17)
    rel = []
    for e in range(ds.n_elements):
        z = rng.integers(0, 3, ds.tree.n_nodes).astype(np.int32)
        rc = rng.uniform(0.1, 0.9)
        a = c32.loglik(e, z, rc, 6.0).sum()
        b = c64.loglik(e, z, rc, 6.0).sum()
        rel.append(abs(a - b) / abs(b))
    rel = np.array(rel)
    assert rel.max() <= TOL_LL, (rel.max(), int(rel.argmax()))
