"""GPU parity of knn_data against the bit-exact FP64 oracle (the reference's
euclidean_distance / correlation_distance restated operation for operation)."""
import os

import numpy as np
import pytest

from mdsctk_gb300 import synth

REF = os.path.join(os.path.dirname(__file__), "golden")


def _recheck_launches(k, centred=0):
    """Launches of the candidate recheck: three stages (candidates, exact
    values, finish) for k + 1 <= 64, plus the block kernel when some rows
    need all their candidates, plus (correlation) the centring of each
    distinct set; one block kernel launch otherwise."""
    return (3 + centred, 4 + centred) if k + 1 <= 64 else (1,)


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


# ---------------------------------------------------------------------------
# tensor-core screen (split BF16, precision "bf16x3"): the recheck makes the
# output bit-identical to the oracle's whatever the screen keeps; these cases
# cover the kernel's tiling edges (row pair tiles of 256, column tiles of
# 128, K-blocks of 32 dimensions, 3 and 4 pipeline stages) and its fallbacks.
@pytest.mark.gpu
@pytest.mark.parametrize("corr", [False, True])
def test_knn_data_tc_vonmises(ctx, oracle, corr):
    x = synth.dihedral_vectors(700, 64, seed=3).astype(np.float64)
    d, i = ctx.knn_data(x, None, 20, correlation=corr, precision="bf16x3")
    st = ctx.stats()
    od, oi = oracle.knn_data(x, None, 20, correlation=corr)
    _check(d, i, od, oi)
    assert st["rows_flagged"] == 0
    # prep, BF16 split, tensor-core screen, recheck
    assert st["launches"] - 3 in _recheck_launches(20, centred=1 if corr else 0)


@pytest.mark.gpu
@pytest.mark.parametrize("nref,nfit,dim,k", [(300, 77, 3, 10), (1000, 513, 100, 25), (129, 255, 32, 7),
                                             (2000, 300, 17, 120)])
def test_knn_data_tc_fit_vs_ref(ctx, oracle, nref, nfit, dim, k):
    rng = np.random.default_rng(nref + dim)
    ref = rng.normal(size=(nref, dim))
    fit = rng.normal(size=(nfit, dim))
    d, i = ctx.knn_data(ref, fit, k, precision="bf16x3")
    st = ctx.stats()
    od, oi = oracle.knn_data(ref, fit, k)
    _check(d, i, od, oi)
    assert st["launches"] - 5 in _recheck_launches(k)  # two preps, two splits, screen, recheck


@pytest.mark.gpu
def test_knn_data_tc_ties_and_duplicates(ctx, oracle):
    """Repeated vectors and zero vectors: exact ties at distance 0 and between
    neighbours; the row guard must send rows whose k+1-th distance equals the
    screen's cut to a wider pass."""
    rng = np.random.default_rng(11)
    base = rng.integers(-3, 4, size=(90, 8)).astype(np.float64)
    x = np.concatenate([base, base, base[:40], np.zeros((30, 8))])
    d, i = ctx.knn_data(x, None, 15, precision="bf16x3")
    od, oi = oracle.knn_data(x, None, 15)
    _check(d, i, od, oi)


@pytest.mark.gpu
def test_knn_data_tc_matches_fp32_screen_large(ctx):
    """5,000 x 64 von Mises vectors, k=32: both screens give the same output
    (each is checked against the oracle at small sizes above)."""
    x = synth.dihedral_vectors(5000, 64, seed=8).astype(np.float64)
    d1, i1 = ctx.knn_data(x, None, 32, precision="bf16x3")
    assert ctx.stats()["rows_flagged"] == 0
    d0, i0 = ctx.knn_data(x, None, 32)
    assert np.array_equal(d1, d0)
    bad = np.argwhere(i1 != i0)
    for r, c in bad:
        assert np.sum(d0[r] == d0[r, c]) >= 2


@pytest.mark.gpu
def test_knn_data_tc_fallback_shapes(ctx, oracle):
    """Shapes outside the tensor-core screen's limits: a dimension above 128
    runs the FP32 screen; a k whose K' exceeds both screens' list sizes (192)
    is rechecked exactly against every reference vector."""
    rng = np.random.default_rng(5)
    x = rng.normal(size=(400, 130))
    d, i = ctx.knn_data(x, None, 9, precision="bf16x3")
    assert ctx.stats()["launches"] - 2 in _recheck_launches(9)  # prep, FP32 screen, recheck
    od, oi = oracle.knn_data(x, None, 9)
    _check(d, i, od, oi)
    x = rng.normal(size=(600, 4))
    for prec in ("bf16x3", "fp32"):
        d, i = ctx.knn_data(x, None, 300, precision=prec)
        st = ctx.stats()
        assert st["launches"] == 2 and st["kprime"] == 0  # prep, exact recheck of every pair
        od, oi = oracle.knn_data(x, None, 300)
        _check(d, i, od, oi)


@pytest.mark.gpu
def test_knn_data_fp32_large_k(ctx, oracle):
    """k = 150: K' is capped at the FP32 screen's pool size (192) and the rows
    still come out exact."""
    rng = np.random.default_rng(6)
    x = rng.normal(size=(1500, 6))
    d, i = ctx.knn_data(x, None, 150)
    assert ctx.stats()["kprime"] == 192
    od, oi = oracle.knn_data(x, None, 150)
    _check(d, i, od, oi)


# launches of the locality order (vec_order.cu): k-means (seed, 6 x assign +
# update, final assign, keys), 2 radix passes of 3, the permutation; for a
# second set assign, keys, sort, permutation; column and row tile geometry,
# coarse bounds, (start tiles over all), threshold seeds, refined bounds,
# (start tiles per segment), rowthr back to the input order
ORDER_LAUNCHES_SAME = 22 + 5 + 1
ORDER_LAUNCHES_FIT = 22 + 9 + 7 + 1


@pytest.mark.gpu
@pytest.mark.parametrize("skip", [False, True])
@pytest.mark.parametrize("fit_rows", [None, 700])
def test_knn_data_tc_pilot_pass(ctx, oracle, fit_rows, skip):
    """9,000 reference vectors (71 column tiles). In input order the screen
    first seeds every row's threshold from 16 tiles (around the diagonal for a
    set against itself, spread over the set for separate fit vectors); in
    locality order each row pair's near segment is screened first instead."""
    rng = np.random.default_rng(21)
    ref = synth.dihedral_vectors(9000, 16, seed=12).astype(np.float64)
    fit = None if fit_rows is None else rng.normal(scale=0.7, size=(fit_rows, 16))
    d, i = ctx.knn_data(ref, fit, 12, precision="bf16x3", skip=skip)
    st = ctx.stats()
    od, oi = oracle.knn_data(ref, fit, 12)
    _check(d, i, od, oi)
    plain = 4 if fit is None else 6  # prep(s), split(s), pilot, screen
    # in locality order: no pilot pass (each row pair's near segment goes first)
    extra = (ORDER_LAUNCHES_SAME if fit is None else ORDER_LAUNCHES_FIT) - 1 if skip else 0
    assert st["launches"] - plain - extra in _recheck_launches(12)


def _sampled(ctx, oracle, ref, fit, k, rows, corr=False):
    """Both tensor-core screens (locality order with tile skipping, and every
    tile in input order) give the same output, and sampled rows match the
    oracle bit for bit."""
    d, i = ctx.knn_data(ref, fit, k, correlation=corr, precision="bf16x3")
    st = ctx.stats()
    d0, i0 = ctx.knn_data(ref, fit, k, correlation=corr, precision="bf16x3", skip=False)
    st0 = ctx.stats()
    assert np.array_equal(d, d0)
    for r, c in np.argwhere(i != i0):
        assert np.sum(d0[r] == d0[r, c]) >= 2
    q = ref if fit is None else fit
    od, oi = oracle.knn_data(ref, q[rows], k, correlation=corr)
    _check(d[rows], i[rows], od, oi)
    return st, st0


@pytest.mark.gpu
def test_knn_data_tc_ordered_mixture(ctx, oracle):
    """20,000 x 64 von Mises mixture vectors against themselves, k = 32: in
    locality order the screen skips most column tiles."""
    x = synth.dihedral_vectors(20_000, 64, seed=31).astype(np.float64)
    st, st0 = _sampled(ctx, oracle, x, None, 32, np.linspace(0, 19_999, 200).astype(int))
    assert st["rows_flagged"] == 0
    assert st["screen_pairs"] < 0.6 * st0["screen_pairs"], (st["screen_pairs"], st0["screen_pairs"])


@pytest.mark.gpu
def test_knn_data_tc_ordered_fit_vs_ref(ctx, oracle):
    """Separate fit vectors (another mixture draw) ordered by the reference
    set's centroids; uneven sizes (12,345 references, 3,001 fit rows)."""
    ref = synth.dihedral_vectors(12_345, 64, seed=32).astype(np.float64)
    fit = synth.dihedral_vectors(3_001, 64, seed=33).astype(np.float64)
    _sampled(ctx, oracle, ref, fit, 20, np.arange(3_001))


@pytest.mark.gpu
def test_knn_data_tc_ordered_duplicates(ctx, oracle):
    """1,500 vectors each present four times (exact ties at distance 0 and
    between neighbours) plus 300 zero vectors."""
    rng = np.random.default_rng(34)
    base = rng.normal(size=(1_500, 24))
    x = np.concatenate([base, base, base, base, np.zeros((300, 24))])[rng.permutation(6_300)]
    _sampled(ctx, oracle, x, None, 10, np.arange(6_300))


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [32, 100])
def test_knn_data_tc_ordered_unstructured(ctx, oracle, dim):
    """Gaussian vectors (no clusters: tiles overlap, little is skipped);
    padded dimensions 32 and 128."""
    x = np.random.default_rng(35 + dim).normal(size=(6_000, dim))
    _sampled(ctx, oracle, x, None, 16, np.arange(0, 6_000, 3))


@pytest.mark.gpu
@pytest.mark.parametrize("k", [90, 100])
def test_knn_data_tc_ordered_large_k(ctx, oracle, k):
    """Locality order at k + 1 = 91 (threshold heaps of 46 per half) and
    k + 1 = 101 (above the heaps' limit: thresholds from list searches)."""
    x = synth.dihedral_vectors(8_000, 64, seed=36).astype(np.float64)
    _sampled(ctx, oracle, x, None, k, np.arange(0, 8_000, 7))


@pytest.mark.gpu
def test_knn_data_tc_ordered_dim96_and_one_fit_row(ctx, oracle):
    """Padded dimension 96 (80 dimensions) in locality order, and a fit set of
    a single vector against 5,000 references."""
    rng = np.random.default_rng(37)
    x = rng.normal(size=(5_000, 80)) + rng.integers(0, 4, size=(5_000, 1)) * 3.0
    _sampled(ctx, oracle, x, None, 12, np.arange(0, 5_000, 5))
    _sampled(ctx, oracle, x, x[1234:1235] + 0.01, 12, np.arange(1))


@pytest.mark.gpu
def test_knn_data_tc_ordered_correlation(ctx, oracle):
    """Correlation metric in locality order (the standardised vectors' tiles
    and bounds): 20,000 x 64 mixture vectors against themselves, k = 32, and
    3,001 separate fit vectors against 12,345 references, k = 20."""
    x = synth.dihedral_vectors(20_000, 64, seed=41).astype(np.float64)
    st, st0 = _sampled(ctx, oracle, x, None, 32, np.linspace(0, 19_999, 200).astype(int), corr=True)
    assert st["screen_pairs"] < st0["screen_pairs"], (st["screen_pairs"], st0["screen_pairs"])
    fit = synth.dihedral_vectors(3_001, 64, seed=42).astype(np.float64)
    _sampled(ctx, oracle, x[:12_345], fit, 20, np.arange(0, 3_001, 3), corr=True)


@pytest.mark.gpu
def test_knn_data_tc_ordered_correlation_offset(ctx, oracle):
    """Correlation of vectors on a large common offset (1e4 + N(0, 0.01^2)):
    the single-pass standard deviation loses digits, so the standardised
    vectors' norms stray from 1 and the bounds' margin grows with them; each
    vector present twice (ties at distance 0)."""
    rng = np.random.default_rng(43)
    base = 1e4 + 0.01 * rng.normal(size=(2_500, 24)) + 0.02 * rng.integers(0, 3, size=(2_500, 1)) * np.arange(24)
    x = np.concatenate([base, base])[rng.permutation(5_000)]
    _sampled(ctx, oracle, x, None, 10, np.arange(0, 5_000, 2), corr=True)
