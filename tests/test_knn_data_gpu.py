"""GPU parity of knn_data against the bit-exact FP64 oracle (the reference's
euclidean_distance / correlation_distance restated operation for operation)."""
import os

import numpy as np
import pytest

from mdsctk_gb300 import synth

REF = os.path.join(os.path.dirname(__file__), "golden")


def _check(d, i, od, oi):
    assert d.shape == od.shape
    # distances are computed in the reference's own arithmetic: bit-identical
    assert np.array_equal(d, od)
    bad = np.argwhere(i != oi)
    for r, c in bad:  # index swaps only among exactly equal distances
        assert np.sum(od[r] == od[r, c]) >= 2


@pytest.mark.gpu
@pytest.mark.parametrize("corr", [False, True])
def test_knn_data_vonmises(ctx, oracle, corr):
    x = synth.dihedral_vectors(700, 64, seed=3).astype(np.float64)
    d, i = ctx.knn_data(x, None, 20, correlation=corr)
    od, oi = oracle.knn_data(x, None, 20, correlation=corr)
    _check(d, i, od, oi)
    assert ctx.stats()["rows_flagged"] == 0


@pytest.mark.gpu
def test_knn_data_fit_vs_ref_and_full(ctx, oracle):
    rng = np.random.default_rng(4)
    ref = rng.normal(size=(300, 3))
    fit = rng.normal(size=(77, 3))
    d, i = ctx.knn_data(ref, fit, 10)
    od, oi = oracle.knn_data(ref, fit, 10)
    _check(d, i, od, oi)
    d, i = ctx.knn_data(ref[:50], fit[:20], 0, sort=False)
    od, oi = oracle.knn_data(ref[:50], fit[:20], 0, sort=False)
    assert np.array_equal(d, od)


@pytest.mark.gpu
@pytest.mark.parametrize("name,dim,k", [("rings", 2, 12), ("swissroll", 3, 12)])
def test_knn_data_reference_fixtures(ctx, oracle, name, dim, k):
    """The reference's own example inputs (examples/*.pts, copied as fixtures)."""
    path = os.path.join(REF, f"{name}.pts")
    x = np.fromfile(path, dtype=np.float64).reshape(-1, dim)
    d, i = ctx.knn_data(x, None, k)
    od, oi = oracle.knn_data(x, None, k)
    _check(d, i, od, oi)
