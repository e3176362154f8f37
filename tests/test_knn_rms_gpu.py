"""GPU parity of knn_rms against the FP64 oracle (tests marked gpu)."""
import numpy as np
import pytest

from mdsctk_gb300 import synth

TOL_A = 1e-4  # 1e-5 nm in the file's Angstrom units


def _check_knn(d, i, od, oi, tol=TOL_A):
    """Distances within tol; indices equal except where the oracle's
    neighbouring distances are within tol of each other (near ties)."""
    assert d.shape == od.shape
    assert np.max(np.abs(d - od)) <= tol, np.max(np.abs(d - od))
    bad = np.argwhere(i != oi)
    for r, c in bad:
        # a swap is legitimate only inside a tie band
        v = od[r, c]
        assert abs(d[r, c] - v) <= tol
        near = np.abs(od[r] - v) <= 2 * tol
        assert near.sum() >= 2, (r, c, i[r, c], oi[r, c], v)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16x3", "fp16x3"])
@pytest.mark.parametrize("n,natoms,k,basins", [(300, 304, 20, 1), (257, 97, 10, 4), (200, 1000, 30, 2)])
def test_knn_rms_self(ctx, oracle, precision, n, natoms, k, basins):
    x = synth.trajectory(n, natoms, seed=n + natoms, basins=basins, dwell=60)
    m = synth.uniform_masses(natoms)
    d, i = ctx.knn_rms(x, None, m, k, precision=precision)
    od, oi = oracle.knn_rms(x, None, m, k)
    _check_knn(d, i, od, oi)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_knn_rms_fit_vs_ref_masses(ctx, oracle, precision):
    rng = np.random.default_rng(1)
    ref = synth.trajectory(220, 60, seed=11, basins=3, dwell=40)
    fit = synth.trajectory(75, 60, seed=12, basins=3, dwell=40)
    m = rng.uniform(1.0, 16.0, size=60).astype(np.float32)
    d, i = ctx.knn_rms(ref, fit, m, 15, precision=precision)
    od, oi = oracle.knn_rms(ref, fit, m, 15)
    _check_knn(d, i, od, oi)


@pytest.mark.gpu
def test_knn_rms_nofit_and_full(ctx, oracle):
    x = synth.trajectory(150, 45, seed=5)
    m = synth.uniform_masses(45)
    d, i = ctx.knn_rms(x, None, m, 12, nofit=True)
    od, oi = oracle.knn_rms(x, None, m, 12, nofit=True)
    _check_knn(d, i, od, oi)
    d, i = ctx.knn_rms(x[:40], x[40:90], m, 0, sort=False)
    od, oi = oracle.knn_rms(x[:40], x[40:90], m, 0, sort=False)
    assert np.max(np.abs(d - od)) <= TOL_A
    assert (i == np.arange(40)[None, :]).all()


@pytest.mark.gpu
def test_knn_rms_k_clamp_and_tiny(ctx, oracle):
    x = synth.trajectory(5, 10, seed=2)
    m = synth.uniform_masses(10)
    d, i = ctx.knn_rms(x, None, m, 50)  # k clamped to 4
    od, oi = oracle.knn_rms(x, None, m, 50)
    assert d.shape == (5, 4)
    _check_knn(d, i, od, oi)
    d, i = ctx.knn_rms(x[:1], None, m, 3)  # one frame: k = 0
    assert d.shape == (1, 0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["bf16x3", "fp16x3"])
def test_knn_rms_tile_skipping_exact(ctx, oracle, precision):
    """Multi-basin data on enough column tiles that the tensor-core screen
    skips tiles by the triangle inequality (pivot pass + main screen): the
    result must still equal the FP64 oracle, self and query sets alike."""
    x = synth.trajectory(2400, 64, seed=77, basins=6, dwell=120, drift_sigma=0.06)
    q = synth.trajectory(300, 64, seed=78, basins=6, dwell=120, drift_sigma=0.06, off_manifold=0.1)
    m = synth.uniform_masses(64)
    for fit in (None, q):
        d, i = ctx.knn_rms(x, fit, m, 20, precision=precision)
        st = ctx.stats()
        assert st["screen_launches"] == 2  # pivot pass + screen
        nf = len(x) if fit is None else len(fit)
        npiv = (len(x) + 39) // 40 if fit is None else (len(x) + 79) // 80
        tiles = ((nf + 39) // 40) * ((len(x) + 79) // 80)
        # pairs computed: the pivot pass plus at least one tile, at most every tile; the
        # trajectory screened against itself skips some
        assert npiv * nf + 3200 <= st["screen_pairs"] <= npiv * nf + tiles * 3200
        if fit is None:
            assert st["screen_pairs"] < npiv * nf + tiles * 3200
        od, oi = oracle.knn_rms(x, fit, m, 20)
        assert np.max(np.abs(d - od)) <= 1e-4
        assert np.mean(i == oi) > 0.999


@pytest.mark.gpu
def test_knn_rms_fp32_tile_skipping_exact(ctx, oracle):
    """The FP32 CUDA-core screen skips tiles of a set screened against itself
    with the same row-tile pivots (its own dense pass over them): fewer pairs
    than every tile, the same result as with skipping off, and the oracle's."""
    x = synth.trajectory(2400, 64, seed=77, basins=6, dwell=120, drift_sigma=0.06)
    m = synth.uniform_masses(64)
    d, i = ctx.knn_rms(x, None, m, 20, precision="fp32")
    st = ctx.stats()
    assert st["screen_launches"] == 2  # pivot pass + screen
    npiv = (len(x) + 39) // 40
    tiles = ((len(x) + 31) // 32) * ((len(x) + 63) // 64)
    assert npiv * len(x) < st["screen_pairs"] < npiv * len(x) + tiles * 2048
    d2, i2 = ctx.knn_rms(x, None, m, 20, precision="fp32", skip=False)
    st2 = ctx.stats()
    assert st2["screen_launches"] == 1 and st2["screen_pairs"] == tiles * 2048
    assert np.array_equal(d, d2) and np.array_equal(i, i2)
    od, oi = oracle.knn_rms(x, None, m, 20)
    assert np.max(np.abs(d - od)) <= 1e-4
    assert np.mean(i == oi) > 0.999


@pytest.mark.gpu
def test_knn_rms_pinned_host_frames(ctx):
    """Page-locked host frames (the chunked upload overlaps the copies with
    the superposition) give the results of ordinary (pageable) host memory,
    for a set against itself and for a separate fit set."""
    import torch

    x = synth.trajectory(3000, 200, seed=5, drift_sigma=0.05)
    m = np.ones(200, np.float32)
    d0, i0 = ctx.knn_rms(x, None, m, 20, precision="bf16x3")
    xp = torch.from_numpy(x).pin_memory()
    d1, i1 = ctx.knn_rms(xp, None, m, 20, precision="bf16x3")
    assert np.array_equal(d0, d1) and np.array_equal(i0, i1)
    f = x[::6].copy()
    d2, i2 = ctx.knn_rms(xp, torch.from_numpy(f).pin_memory(), m, 20, precision="bf16x3")
    d3, i3 = ctx.knn_rms(x, f, m, 20, precision="bf16x3")
    assert np.array_equal(d2, d3) and np.array_equal(i2, i3)


@pytest.mark.gpu
def test_knn_rms_pinned_staged_chunks(ctx):
    """Page-locked frames of a set against itself take the staged path (the
    pivots' frames gathered first; each upload chunk superposed, split and
    bounded against the pivots as it lands): several chunks and a partial
    last row tile give the unstaged path's results bit for bit."""
    import torch

    x = synth.trajectory(20_017, 64, seed=15, basins=4, dwell=300.0, drift_sigma=0.05)
    m = np.ones(64, np.float32)
    d0, i0 = ctx.knn_rms(x, None, m, 16, precision="bf16x3")
    assert ctx.stats()["screen_launches"] == 2
    xp = torch.from_numpy(x).pin_memory()
    d1, i1 = ctx.knn_rms(xp, None, m, 16, precision="bf16x3")
    st = ctx.stats()
    assert st["screen_launches"] == 2 and st["rows_flagged"] == 0
    assert np.array_equal(d0, d1) and np.array_equal(i0, i1)
