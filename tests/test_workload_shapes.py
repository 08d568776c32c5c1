"""The synthetic workloads have the shapes of the configurations they stand in
for (taxa, total tree length, targets, element-length distribution, the
accelerated share), so that the benchmark's lines measure those
configurations.  CPU only."""
import numpy as np
import pytest

from phyloacc_gb300 import synth


def _lengths(ds):
    return np.asarray(ds.lengths, dtype=np.int64)


def test_twelve_taxa_configuration():
    ds = synth.make_dataset("st12", seed=0)
    assert ds.tree.n_nodes == 23 and ds.n_elements == 100
    assert abs(ds.tree.distances.sum() - 1.2) < 1e-6
    L = _lengths(ds)
    assert L.min() >= 100 and L.max() <= 300
    assert int(np.sum(ds.accelerated)) == 20
    assert len(ds.target) == 3


@pytest.mark.parametrize("kind,clip", [("st43", 2000), ("st43_serve", 5000)])
def test_forty_three_taxa_configurations(kind, clip):
    ds = synth.make_dataset(kind, n_elements=1500, seed=3)
    assert ds.tree.n_nodes == 85
    assert abs(ds.tree.distances.sum() - 2.5) < 1e-6
    assert len(ds.target) == 8
    L = _lengths(ds)
    assert L.min() >= 50 and L.max() <= clip
    # log-normal, median 250 bp, sigma 0.6
    assert abs(np.median(L) - 250) < 20
    assert abs(np.std(np.log(L)) - 0.6) < 0.05
    assert 0.07 < np.mean(ds.accelerated) < 0.13


def test_stress_set_configuration():
    base = synth.make_dataset("st43", n_elements=10, seed=3)
    ds = synth.make_dataset("st43_stress", n_elements=10, seed=3)
    assert np.all(_lengths(ds) == 2000)
    np.testing.assert_allclose(ds.tree.distances, 5 * base.tree.distances, rtol=1e-6)
    assert np.all(ds.r2[np.asarray(ds.accelerated, bool)] == 6.0)


def test_gbgc_configuration():
    ds = synth.make_dataset("gbgc120", n_elements=300, seed=3)
    assert ds.tree.n_nodes == 239
    assert abs(ds.tree.distances.sum() - 4.0) < 1e-6
    assert len(ds.target) == 20
    L = _lengths(ds)
    assert L.min() >= 50 and L.max() <= 3000
    assert abs(np.median(L) - 300) < 30
