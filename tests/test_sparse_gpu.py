"""GPU parity of make_sysparse / make_gesparse / decomp_sparse /
decomp_sparse_nystrom against the oracle (bit-exact for the assembly;
eigenvalues 1e-6 relative, eigenvectors 1e-5 up to sign)."""
import numpy as np
import pytest

from mdsctk_gb300 import synth


def _knn(oracle, x, k):
    return oracle.knn_data(x, None, k)


@pytest.mark.gpu
@pytest.mark.parametrize("k", [None, 3])
def test_sysparse_random_with_duplicates(ctx, oracle, k):
    rng = np.random.default_rng(11)
    n, maxk = 500, 7
    idx = rng.integers(0, n, size=(n, maxk)).astype(np.int32)
    dist = rng.uniform(0, 2, size=(n, maxk))
    a = ctx.sysparse(dist, idx, k)
    b = oracle.sysparse(dist, idx, k)
    for u, v in zip(a[1:], b[1:]):
        assert np.array_equal(u, v)


@pytest.mark.gpu
def test_sysparse_knn_graph_and_edge_cases(ctx, oracle):
    x = synth.dihedral_vectors(900, 8, seed=2).astype(np.float64)
    d, i = oracle.knn_data(x, None, 12)
    a = ctx.sysparse(d, i)
    b = oracle.sysparse(d, i)
    for u, v in zip(a[1:], b[1:]):
        assert np.array_equal(u, v)
    # empty and negative-index inputs
    e = ctx.sysparse(np.zeros((0, 3)), np.zeros((0, 3), np.int32))
    assert e[0] == 0 and e[1].tolist() == [0]
    idx = np.array([[1, -1], [0, 2], [1, 0]], np.int32)
    a = ctx.sysparse(np.ones((3, 2)), idx)
    assert a[1][-1] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("sym", [False, True])
def test_gesparse(ctx, oracle, sym):
    rng = np.random.default_rng(3)
    m, n, k = 200, 300, 6
    idx = rng.integers(0, n, size=(m, k)).astype(np.int32)
    dist = rng.uniform(0, 2, size=(m, k))
    a = ctx.gesparse(dist, idx, symmetric=sym)
    b = oracle.gesparse(dist, idx, symmetric=sym)
    for u, v in zip(a[1:], b[1:]):
        assert np.array_equal(u, v)


def _align_sign(v, ref):
    return v * (1.0 if np.dot(v, ref) >= 0 else -1.0)


@pytest.mark.gpu
@pytest.mark.parametrize("ncv,tol", [(0, 0.0), (40, 1e-8)])
def test_decomp_sparse_vs_arpack(ctx, oracle, ncv, tol):
    rng = np.random.default_rng(5)
    # three well-separated clusters -> a connected graph with a clear gap
    x = np.concatenate([rng.normal(size=(300, 3)) + c for c in ([0, 0, 0], [4, 0, 0], [0, 4, 0])])
    d, i = oracle.knn_data(x, None, 15)
    n, pcol, irow, val = oracle.sysparse(d, i)
    sigma = float(np.median(d))
    nev = 8
    w, V, res, nconv = ctx.decomp_sparse(n, pcol, irow, val, sigma, nev, ncv=ncv, tol=tol)
    wo, Vo, reso = oracle.decomp_sparse(n, pcol, irow, val, sigma, nev,
                                        ncv=ncv if ncv else None, tol=tol)
    assert nconv == nev
    assert np.allclose(w, wo, rtol=1e-6, atol=1e-9)
    for x in range(nev):
        gap = min(abs(w[x] - w[y]) for y in range(nev) if y != x)
        if gap > 1e-6:
            assert np.max(np.abs(_align_sign(V[x], Vo[x]) - Vo[x])) < 1e-5, x
    assert np.all(res < 1e-6)


@pytest.mark.gpu
def test_decomp_degenerate_spectrum_subspace(ctx, oracle):
    """Disconnected components: eigenvalue 1 repeated; compare subspaces."""
    rng = np.random.default_rng(6)
    x = np.concatenate([rng.normal(size=(200, 2)), rng.normal(size=(200, 2)) + 100.0])
    d, i = oracle.knn_data(x, None, 10)
    n, pcol, irow, val = oracle.sysparse(d, i)
    w, V, res, nconv = ctx.decomp_sparse(n, pcol, irow, val, 1.0, 4)
    wo, Vo, _ = oracle.decomp_sparse(n, pcol, irow, val, 1.0, 4)
    assert np.allclose(w, wo, rtol=1e-6, atol=1e-9)
    Q1, _ = np.linalg.qr(V[:2].T)
    Q2, _ = np.linalg.qr(Vo[:2].T)
    s = np.linalg.svd(Q1.T @ Q2, compute_uv=False)
    assert np.min(s) > 1 - 1e-8


@pytest.mark.gpu
def test_nystrom_extension(ctx, oracle):
    rng = np.random.default_rng(8)
    land = np.concatenate([rng.normal(size=(250, 2)), rng.normal(size=(250, 2)) + 5])
    qry = np.concatenate([rng.normal(size=(60, 2)), rng.normal(size=(60, 2)) + 5])
    d, i = oracle.knn_data(land, None, 12)
    n, pcol, irow, val = oracle.sysparse(d, i)
    dq, iq = oracle.knn_data(land, qry, 12)
    m, pb, ib, vb = oracle.gesparse(dq, iq)
    sigma = 1.0
    w, V, E, res, nconv = ctx.decomp_sparse_nystrom(n, pcol, irow, val, m, pb, ib, vb, sigma, 5)
    wo, Vo, _ = oracle.decomp_sparse(n, pcol, irow, val, sigma, 5)
    A, dinv = oracle.affinity(n, pcol, irow, val, sigma)
    Bo = oracle.affinity_nystrom(m, pb, ib, vb, sigma, dinv)
    assert np.allclose(w, wo, rtol=1e-6)
    for x in range(5):
        ext_o = oracle.sp_dgemv(m, pb, ib, Bo, V[x] / w[x])  # the extension of this run's vector
        assert np.max(np.abs(E[x] - ext_o)) < 1e-10


def _rings_graph(oracle, k=20, keep=12):
    import os

    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    x = np.fromfile(os.path.join(gold, "rings.pts"), np.float64).reshape(-1, 2)
    d, i = oracle.knn_data(x, None, k)
    return oracle.sysparse(d, i, keep)


@pytest.mark.gpu
@pytest.mark.parametrize("ka", [1, 7, 12, 40])
def test_auto_sigmas_mean_bit_exact(ctx, oracle, ka):
    """k-sigma means: the first ka entries in neighbour-index order, sorted,
    summed in ascending order (bit-exact), lists shorter than ka included."""
    n, pcol, irow, val = _rings_graph(oracle)
    w, V, res, nconv, sig = ctx.auto_decomp_sparse(n, pcol, irow, val, ka, 4)
    osig = oracle.auto_sigmas(n, pcol, irow, val, ka)
    assert np.array_equal(sig, osig)
    wo, Vo, _, _ = oracle.auto_decomp_sparse(n, pcol, irow, val, ka, 4)
    assert np.allclose(w, wo, rtol=1e-6, atol=1e-9)
    assert np.max(res) < 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("K", [3.0, 7.5, 12.0])
def test_auto_sigmas_entropic(ctx, oracle, K):
    n, pcol, irow, val = _rings_graph(oracle)
    w, V, res, nconv, sig = ctx.auto_decomp_sparse(n, pcol, irow, val, 12, 5, perplexity=K)
    wo, Vo, _, osig = oracle.auto_decomp_sparse(n, pcol, irow, val, 12, 5, perplexity=K)
    # same roots, different warm starts: agreement to the root-finding tolerance
    assert np.allclose(sig, osig, rtol=1e-8)
    assert np.allclose(w, wo, rtol=1e-6, atol=1e-9)
    _same_subspaces(wo, V, Vo)


def _same_subspaces(w, V, Vo, gap=1e-5):
    """Eigenvectors agree up to rotation within groups of eigenvalues closer
    than `gap` (sigmas that differ at 1e-10 rotate nearly degenerate pairs);
    the group holding the last eigenvalue is skipped (its partners beyond nev
    are unknown)."""
    groups, cur = [], [0]
    for x in range(1, len(w)):
        if abs(w[x] - w[x - 1]) < gap * max(1.0, abs(w[x])):
            cur.append(x)
        else:
            groups.append(cur)
            cur = [x]
    for g in groups:  # `cur` (the last group) is not compared
        Q1, _ = np.linalg.qr(V[g].T)
        Q2, _ = np.linalg.qr(Vo[g].T)
        assert np.min(np.linalg.svd(Q1.T @ Q2, compute_uv=False)) > 1 - 1e-6


@pytest.mark.gpu
def test_auto_sigmas_rejects_short_lists(ctx, oracle):
    from mdsctk_gb300 import MdsError

    n, pcol, irow, val = _rings_graph(oracle, keep=3)
    with pytest.raises(MdsError):  # every list holds >= 3, some < 30: the reference reads past them
        ctx.auto_decomp_sparse(n, pcol, irow, val, 30, 3, perplexity=5.0)
    with pytest.raises(MdsError):  # ceil(K) > k-sigma
        ctx.auto_decomp_sparse(n, pcol, irow, val, 3, 3, perplexity=5.0)


@pytest.mark.gpu
def test_auto_nystrom(ctx, oracle):
    rng = np.random.default_rng(8)
    land = np.concatenate([rng.normal(size=(250, 2)), rng.normal(size=(250, 2)) + 5])
    qry = np.concatenate([rng.normal(size=(60, 2)), rng.normal(size=(60, 2)) + 5])
    d, i = oracle.knn_data(land, None, 12)
    n, pcol, irow, val = oracle.sysparse(d, i)
    dq, iq = oracle.knn_data(land, qry, 12)
    m, pb, ib, vb = oracle.gesparse(dq, iq)
    w, V, E, res, nconv, sig = ctx.auto_decomp_sparse_nystrom(n, pcol, irow, val, m, pb, ib, vb, 8, 5)
    osig = oracle.auto_sigmas(n, pcol, irow, val, 8)
    assert np.array_equal(sig, osig)
    _, d_a = oracle.affinity_auto(n, pcol, irow, val, osig)
    Bo = oracle.affinity_nystrom_auto(m, pb, ib, vb, osig, d_a)
    Eo = oracle.nystrom_extend(w, V, m, pb, ib, Bo)
    assert np.max(np.abs(E - Eo)) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("nev", [3, 5])
def test_decomp_triple_eigenvalue(ctx, oracle, nev):
    """Three disconnected basins: eigenvalue 1 three times, with 0.99999996,
    0.9999 and 0.9996 just below. Lanczos from one start vector finds one
    copy; the completion on the deflated operator must find the others,
    also when nev leaves no room beyond the three copies."""
    from mdsctk_gb300 import synth

    land = synth.trajectory(900, 64, seed=31, basins=3, dwell=150)
    m = synth.uniform_masses(64)
    d, i = oracle.knn_rms(land, None, m, 16)
    sigma = float(np.median(d))
    n, pcol, irow, val = oracle.sysparse(d, i)
    exact = np.linalg.eigvalsh(oracle.dense_affinity(n, pcol, irow, val, sigma))[::-1][:nev]
    assert np.sum(np.abs(exact - 1.0) < 1e-12) == 3
    w, V, res, nconv = ctx.decomp_sparse(n, pcol, irow, val, sigma, nev)
    assert np.allclose(w, exact, rtol=1e-6), (w, exact)
    assert np.max(np.abs(V @ V.T - np.eye(nev))) < 1e-10
    assert np.max(res) < 1e-8
