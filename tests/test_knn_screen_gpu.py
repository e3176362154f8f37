"""GPU tests of the knn_rms candidate screen itself (lower-bound property,
completeness of the kept candidates, tightness), through the diagnostic
entry point mds_knn_rms_screen, against the FP64 oracle."""
import numpy as np
import pytest

from mdsctk_gb300 import synth


def _exact_d2(oracle, x, m):
    d, _ = oracle.knn_rms(x, None, m, 0, sort=False)
    return (d / 10.0) ** 2  # Angstrom -> nm, squared


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16x3", "fp16x3"])
@pytest.mark.parametrize("n,natoms,basins", [(320, 304, 4), (240, 1000, 8), (100, 37, 2)])
def test_screen_lower_bound_and_completeness(ctx, oracle, precision, n, natoms, basins):
    x = synth.trajectory(n, natoms, seed=7 * n + natoms, basins=basins, dwell=60, drift_sigma=0.08)
    m = synth.uniform_masses(natoms)
    kp = 64
    lb, idx, cnt = ctx.knn_rms_screen(x, None, m, kp, precision=precision)
    ex = _exact_d2(oracle, x, m)
    assert (cnt == kp).all()
    rows = np.arange(n)[:, None]
    exact_c = ex[rows, idx]
    # lower bound (allow float rounding of the exact value itself)
    assert np.all(lb <= exact_c * (1 + 1e-6) + 1e-9), np.max(lb - exact_c)
    # tight: the bound is close to the exact value for the kept pairs
    gap = exact_c - lb
    assert np.median(gap) < 1e-3, np.median(gap)
    # complete: every pair whose exact value is below the row's threshold is kept
    tau = lb[:, -1]
    for r in range(n):
        must = np.nonzero(ex[r] < tau[r])[0]
        assert set(must.tolist()) <= set(idx[r].tolist()), r


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16x3", "fp16x3"])
def test_screen_lower_bound_off_trajectory_queries(ctx, oracle, precision):
    """Queries off the landmarks' trajectory (distances concentrated, frames
    far from the template): the guarded values stay lower bounds and the
    kept set is complete."""
    land = synth.trajectory(3000, 304, seed=5, basins=16, dwell=100.0)
    qry = synth.trajectory(48, 304, seed=6, basins=16, dwell=100.0, off_manifold=0.2, off_sigma=0.3)
    m = synth.uniform_masses(304)
    lb, idx, cnt = ctx.knn_rms_screen(land, qry, m, 128, precision=precision)
    d, _ = oracle.knn_rms(land, qry, m, 0, sort=False)
    ex = (d / 10.0) ** 2
    rows = np.arange(len(qry))[:, None]
    assert np.all(lb <= ex[rows, idx] * (1 + 1e-6) + 1e-9), np.max(lb - ex[rows, idx])
    tau = lb[:, -1]
    for r in range(len(qry)):
        assert set(np.nonzero(ex[r] < tau[r])[0].tolist()) <= set(idx[r].tolist()), r


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_knn_rms_no_flagged_rows(ctx, oracle, precision):
    """On well-conditioned multi-basin data the guard holds on the first pass."""
    x = synth.trajectory(600, 1000, seed=99, basins=8, dwell=100, drift_sigma=0.08)
    m = synth.uniform_masses(1000)
    d, i = ctx.knn_rms(x, None, m, 30, precision=precision)
    st = ctx.stats()
    assert st["rows_flagged"] == 0, st
    od, oi = oracle.knn_rms(x, None, m, 30)
    assert np.max(np.abs(d - od)) <= 1e-4


def _keymat(S):
    sxx, sxy, sxz, syx, syy, syz, szx, szy, szz = S
    return np.array([[sxx + syy + szz, syz - szy, szx - sxz, sxy - syx],
                     [syz - szy, sxx - syy - szz, sxy + syx, szx + sxz],
                     [szx - sxz, sxy + syx, -sxx + syy - szz, syz + szy],
                     [sxy - syx, szx + sxz, syz + szy, -sxx - syy + szz]])


def _sym(r, o):
    return np.array([[r[o], r[o + 3], r[o + 4]], [r[o + 3], r[o + 1], r[o + 5]], [r[o + 4], r[o + 5], r[o + 2]]],
                    dtype=np.float64)


@pytest.mark.gpu
@pytest.mark.parametrize("nofit", [False, True])
def test_superposition_records(ctx, oracle, nofit):
    """Deviations and records reproduce every pair's RMSD through the
    decomposition S_ij = M0 + U_i + U_j^T + G_ij the screen relies on."""
    n, na = 40, 97
    x = synth.trajectory(n, na, seed=21, basins=3, dwell=10)
    rng = np.random.default_rng(2)
    m = rng.uniform(1, 16, na).astype(np.float32)
    dev, rec = ctx.knn_rms_superpose(x, m, nofit=nofit)
    assert np.all(np.isfinite(dev)) and np.all(np.isfinite(rec))
    assert np.all(dev[:, :, na:] == 0)
    a = dev[:, :, :na].astype(np.float64)
    r = rec.astype(np.float64)
    assert np.allclose(r[:, 15], (a ** 2).sum((1, 2)), rtol=1e-5)
    full, _ = oracle.knn_rms(x, None, m, 0, sort=False, nofit=nofit)
    ex = (full / 10.0) ** 2
    trM0 = r[0, 0:3].sum() - r[0, 6:9].sum()
    E = trM0 + 2 * r[:, 6:9].sum(1) + r[:, 15]
    for i in range(0, n, 7):
        for j in range(n):
            G = a[i] @ a[j].T  # G[c, d] = sum_a a_i^c a_j^d
            if nofit:
                d2 = r[i, 15] + r[j, 15] - 2 * np.trace(G)
            else:
                b = r[i, 12:15] - r[j, 12:15]
                A = 0.5 * np.array([[0, b[2], -b[1]], [-b[2], 0, b[0]], [b[1], -b[0], 0]])
                S = _sym(r[i], 0) + _sym(r[j], 6) + G + A
                lam = np.linalg.eigvalsh(_keymat(S.ravel()))[-1]
                d2 = E[i] + E[j] - 2 * lam
            assert abs(d2 - ex[i, j]) < 2e-5 * (1 + ex[i, j]), (i, j, d2, ex[i, j])
