"""knn_data_sparse and contact_profile on the GPU against the oracle (the
reference's euclidean_distance_sparse walk and contact test restated), and
the two drop-in tools end to end, file for file."""
import os
import subprocess

import numpy as np
import pytest


def _vectors(rng, n, dim, density, sort=True, dup=False):
    vecs = []
    for _ in range(n):
        m = rng.binomial(dim, density)
        ii = rng.choice(dim, m, replace=False)
        if sort:
            ii = np.sort(ii)
        if dup and m > 2:
            ii[-1] = ii[-2]  # a repeated index: the walk decides what it means
        vecs.append((ii.astype(np.int32), rng.normal(size=m)))
    return vecs


def _check(d, i, od, oi):
    assert d.shape == od.shape
    assert np.array_equal(d, od)  # the reference's FP64 walk: bit-identical
    for r, c in np.argwhere(i != oi):  # index swaps only among equal distances
        assert np.sum(od[r] == od[r, c]) >= 2


@pytest.mark.gpu
@pytest.mark.parametrize("k", [1, 7, 40])
def test_knn_data_sparse_self(ctx, oracle, k):
    rng = np.random.default_rng(k)
    vecs = _vectors(rng, 1500, 400, 0.05)
    vecs[3] = (np.zeros(0, np.int32), np.zeros(0))  # an empty vector
    vecs[9] = vecs[10]  # a duplicate: distance 0, a tie
    ref = oracle.csr(vecs)
    d, i = ctx.knn_data_sparse(ref, None, k)
    od, oi = oracle.knn_data_sparse(ref, None, k)
    _check(d, i, od, oi)


@pytest.mark.gpu
def test_knn_data_sparse_fit_full_and_unsorted(ctx, oracle):
    """Separate fit vectors, the full-row mode, unsorted and repeated indices
    (the walk is the reference's, whatever the order), long fit vectors read
    from global memory, and more than one chunk of 1,024 references."""
    rng = np.random.default_rng(5)
    ref = oracle.csr(_vectors(rng, 2300, 300, 0.1, sort=False, dup=True))
    fit_v = _vectors(rng, 70, 300, 0.1)
    fit_v[0] = (np.arange(2500, dtype=np.int32), rng.normal(size=2500))  # beyond the shared-memory copy
    fit = oracle.csr(fit_v)
    d, i = ctx.knn_data_sparse(ref, fit, 12)
    od, oi = oracle.knn_data_sparse(ref, fit, 12)
    _check(d, i, od, oi)
    d, i = ctx.knn_data_sparse(ref, fit, 0, sort=False)
    od, oi = oracle.knn_data_sparse(ref, fit, 0, sort=False)
    assert np.array_equal(d, od) and np.array_equal(i, oi)


@pytest.mark.gpu
def test_contact_profile(ctx, oracle):
    """Random frames plus pairs placed within 1e-6 of the cutoff, so both the
    FP32 decision and the exact (reference arithmetic) path are exercised."""
    rng = np.random.default_rng(3)
    nf, na = 40, 120
    x = rng.uniform(0, 3.0, size=(nf, na, 3)).astype(np.float32)
    eps = 9.0
    for f in range(nf):  # atom 60 at exactly ~eps/10 nm from atom 0 along x, give or take a few ulps
        x[f, 60] = x[f, 0] + np.float32(eps / 10.0 * (1.0 + (f - 20) * 1e-7)) * np.array([1, 0, 0], np.float32)
    g1 = np.arange(0, 50, dtype=np.int32)
    g2 = np.arange(55, 120, dtype=np.int32)
    off, idx = ctx.contact_profile(x, g1, g2, eps)
    ooff, oidx = oracle.contact_profile(x, g1, g2, eps)
    assert np.array_equal(off, ooff)
    assert np.array_equal(idx, oidx)


def _run(bindir, tmp, name, *args, stdin=None):
    r = subprocess.run([os.path.join(bindir, name), *args], cwd=tmp, capture_output=True, text=True, input=stdin)
    assert r.returncode == 0, (name, r.stdout, r.stderr)
    return r.stdout


@pytest.mark.gpu
def test_sparse_tools(ctx, oracle, tmp_path):
    """contact_profile (.pdb topology, raw frames, .ndx groups chosen on
    standard input) -> knn_data_sparse, file for file against the oracle."""
    from mdsctk_gb300 import build

    build.build()
    rng = np.random.default_rng(11)
    nf, na = 60, 30
    x = rng.uniform(0, 2.0, size=(nf, na, 3)).astype(np.float32)
    x.tofile(tmp_path / "traj.raw")
    with open(tmp_path / "top.pdb", "w") as f:
        for a in range(na):
            f.write("ATOM  %5d  CA  ALA A%4d    %8.3f%8.3f%8.3f  1.00  0.00           C\n"
                    % (a + 1, a + 1, *(10 * x[0, a])))
    with open(tmp_path / "groups.ndx", "w") as f:
        f.write("[ first ]\n" + " ".join(str(a + 1) for a in range(0, 12)) + "\n")
        f.write("[ second ]\n" + " ".join(str(a + 1) for a in range(15, 30)) + "\n")
    _run(build.BINDIR, tmp_path, "contact_profile", "-p", "top.pdb", "-x", "traj.raw", "-n", "groups.ndx",
         "-e", "8.0", stdin="0\n1\n")
    ooff, oidx = oracle.contact_profile(x, np.arange(0, 12), np.arange(15, 30), 8.0)
    ib = np.fromfile(tmp_path / "reference.svi", np.int32)
    db = np.fromfile(tmp_path / "reference.svd", np.float64)
    want_i = []
    for f in range(nf):
        n = ooff[f + 1] - ooff[f]
        want_i.append(np.int32(n))
        want_i.extend(oidx[ooff[f]:ooff[f + 1]])
    assert np.array_equal(ib, np.array(want_i, np.int32))
    assert np.array_equal(db, np.ones(ooff[-1]))
    _run(build.BINDIR, tmp_path, "knn_data_sparse", "-k", "5")
    vecs = [(oidx[ooff[f]:ooff[f + 1]], np.ones(ooff[f + 1] - ooff[f])) for f in range(nf)]
    od, oi = oracle.knn_data_sparse(oracle.csr(vecs), None, 5)
    d = np.fromfile(tmp_path / "distances.dat", np.float64).reshape(nf, 5)
    i = np.fromfile(tmp_path / "indices.dat", np.int32).reshape(nf, 5)
    _check(d, i, od, oi)


@pytest.mark.gpu
@pytest.mark.parametrize("fit_rows,k", [(None, 9), (150, 33)])
def test_knn_data_sparse_binary(ctx, oracle, fit_rows, k):
    """Binary vectors (values 1.0, ascending unique indices: contact maps) take
    the bit-set popcount path; distances stay bit-identical to the walk.
    Repeated vectors make ties at distance 0 and between neighbours."""
    rng = np.random.default_rng(17 + k)
    n, dim = 1300, 3000

    def binvec(m):
        ii = np.sort(rng.choice(dim, m, replace=False)).astype(np.int32)
        return ii, np.ones(m)

    vecs = [binvec(int(rng.integers(0, 200))) for _ in range(n)]
    for a in range(0, 60, 3):
        vecs[a + 1] = vecs[a]
    vecs[5] = (np.zeros(0, np.int32), np.zeros(0))
    ref = oracle.csr(vecs)
    fit = None if fit_rows is None else oracle.csr([binvec(int(rng.integers(1, 200))) for _ in range(fit_rows)])
    d, i = ctx.knn_data_sparse(ref, fit, k)
    st = ctx.stats()
    od, oi = oracle.knn_data_sparse(ref, fit, k)
    _check(d, i, od, oi)
    assert st["launches"] == (2 if fit is None else 3)  # bit sets (per set) + popcount tiles
