"""CPU tests of the oracle (the FP64 restatement used as the checker):
cross-checks against independent implementations, RMSD properties, the
reference's ordering/clamping semantics, and the committed golden vectors."""
import os

import numpy as np
import pytest

from mdsctk_gb300 import synth

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def traj():
    return synth.trajectory(60, 40, seed=3, basins=2, dwell=20)


def test_rmsd_matches_scipy_kabsch(oracle, traj):
    from scipy.spatial.transform import Rotation

    m = synth.uniform_masses(40)
    c = oracle.center(traj, m)
    for i, j in [(0, 1), (3, 40), (10, 59)]:
        r = oracle.rmsd(c[i], c[j], m)
        _, rssd = Rotation.align_vectors(c[j].astype(np.float64), c[i].astype(np.float64))
        assert abs(r - rssd / np.sqrt(40)) < 1e-10


def test_rmsd_port_matches_fp64(oracle, traj):
    rng = np.random.default_rng(0)
    m = rng.uniform(1, 16, 40).astype(np.float32)
    c = oracle.center(traj, m)
    for i, j in [(0, 1), (5, 33), (12, 50)]:
        assert abs(oracle.rmsd_port(c[j], c[i], m) - oracle.rmsd(c[i], c[j], m)) < 1e-6


def test_rmsd_invariances(oracle, traj):
    m = synth.uniform_masses(40)
    c = oracle.center(traj, m)
    a, b = c[2], c[17]
    r = oracle.rmsd(a, b, m)
    assert oracle.rmsd(a, a, m) < 1e-6
    assert abs(oracle.rmsd(b, a, m) - r) < 1e-12
    th = 0.7
    R = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    b2 = (b.astype(np.float64) @ R.T + np.array([1.0, -2.0, 0.5])).astype(np.float32)
    b2c = oracle.center(b2[None], m)[0]
    assert abs(oracle.rmsd(a, b2c, m) - r) < 1e-6
    # no-fit RMSD is an upper bound of the fitted one
    assert oracle.rmsd(a, b, m, nofit=True) >= r - 1e-12


def test_knn_rms_semantics(oracle, traj):
    m = synth.uniform_masses(40)
    d, i = oracle.knn_rms(traj, None, m, 5)
    full, _ = oracle.knn_rms(traj, None, m, 0, sort=False)
    for r in range(traj.shape[0]):
        order = np.lexsort((np.arange(full.shape[1]), full[r]))
        assert np.array_equal(i[r], order[1:6])  # k+1 smallest, position 0 dropped
        assert np.allclose(d[r], full[r, order[1:6]])
    # k clamp (knn_rms.cpp:224-225)
    d, i = oracle.knn_rms(traj[:4], None, m, 10)
    assert d.shape == (4, 3)


def test_knn_rms_port_agrees(oracle, traj):
    m = synth.uniform_masses(40)
    d, i = oracle.knn_rms(traj, None, m, 6)
    dp, ip = oracle.knn_rms_port(traj, None, m, 6, blksize=7)
    assert np.max(np.abs(d - dp)) < 1e-4


def test_knn_data_matches_numpy(oracle):
    rng = np.random.default_rng(1)
    x = rng.normal(size=(80, 7))
    d, i = oracle.knn_data(x, None, 6)
    D = np.sqrt(((x[:, None, :] - x[None, :, :]) ** 2).sum(-1))
    for r in range(80):
        order = np.lexsort((np.arange(80), D[r]))
        assert np.array_equal(i[r], order[1:7])
        assert np.allclose(d[r], D[r, order[1:7]], rtol=0, atol=1e-13)
    dc, ic = oracle.knn_data(x, None, 6, correlation=True)
    C = np.corrcoef(x)
    Dc = np.sqrt(np.maximum(0, (1 - C) / 2))
    for r in range(80):
        assert np.allclose(np.sort(Dc[r])[1:7], dc[r], atol=1e-7)


@pytest.mark.parametrize("name,dim,k", [("rings", 2, 12), ("swissroll", 3, 12)])
def test_knn_data_golden(oracle, name, dim, k):
    x = np.fromfile(os.path.join(GOLD, name + ".pts"), dtype=np.float64).reshape(-1, dim)
    g = np.load(os.path.join(GOLD, f"knn_data_{name}.npz"))
    d, i = oracle.knn_data(x, None, k)
    assert np.array_equal(d, g["d"]) and np.array_equal(i, g["i"])


def _sysparse_py(dist, idx, k):
    """Dictionary restatement of make_sysparse.cpp:245-313 (put overwrites)."""
    edges = {}
    n = dist.shape[0]
    for r in range(n):
        for x in range(k):
            j = int(idx[r, x])
            if r < j:
                edges[(r, j)] = dist[r, x]
            if j < r:
                edges[(j, r)] = dist[r, x]
    keys = sorted(edges)
    pcol, irow, val = [0], [], []
    p = 0
    for c in range(n):
        while p < len(keys) and keys[p][0] == c:
            irow.append(keys[p][1])
            val.append(edges[keys[p]])
            p += 1
        pcol.append(len(irow))
    return np.array(pcol), np.array(irow), np.array(val)


def test_sysparse_semantics(oracle):
    rng = np.random.default_rng(5)
    n, maxk = 50, 6
    idx = rng.integers(0, n, size=(n, maxk)).astype(np.int32)  # self and duplicate entries included
    dist = rng.uniform(0, 3, size=(n, maxk))
    for k in (maxk, 3):
        nn, pcol, irow, val = oracle.sysparse(dist, idx, k)
        p2, i2, v2 = _sysparse_py(dist, idx, k)
        assert np.array_equal(pcol, p2) and np.array_equal(irow, i2) and np.array_equal(val, v2)
        # strictly lower triangle: row > column
        cols = np.repeat(np.arange(n), np.diff(pcol))
        assert np.all(irow > cols)


def test_sysparse_negative_index_blocks_cursor(oracle):
    idx = np.array([[1, -1], [0, 2], [1, 0]], np.int32)
    dist = np.ones((3, 2))
    n, pcol, irow, val = oracle.sysparse(dist, idx)
    assert pcol[-1] == 0  # the cursor never leaves the key with from = -1


def test_affinity_and_symv_match_dense(oracle):
    rng = np.random.default_rng(7)
    x = rng.normal(size=(40, 3))
    d, i = oracle.knn_data(x, None, 6)
    n, pcol, irow, val = oracle.sysparse(d, i)
    A, dinv = oracle.affinity(n, pcol, irow, val, 0.8)
    W = np.zeros((n, n))
    for c in range(n):
        for p in range(pcol[c], pcol[c + 1]):
            w = np.exp(-val[p] ** 2 / (2 * 0.8 ** 2))
            W[irow[p], c] = W[c, irow[p]] = w
    deg = W.sum(1)
    Wn = W / np.sqrt(deg)[:, None] / np.sqrt(deg)[None, :]
    M = oracle.dense_affinity(n, pcol, irow, val, 0.8)
    assert np.allclose(M, Wn, atol=1e-14)
    v = rng.normal(size=n)
    assert np.allclose(oracle.sp_dsymv(n, pcol, irow, A, v), Wn @ v, atol=1e-13)


def test_decomp_oracle_vs_dense(oracle):
    rng = np.random.default_rng(9)
    x = np.concatenate([rng.normal(size=(60, 2)), rng.normal(size=(60, 2)) + 6])
    d, i = oracle.knn_data(x, None, 8)
    n, pcol, irow, val = oracle.sysparse(d, i)
    w, V, res = oracle.decomp_sparse(n, pcol, irow, val, 1.0, 4)
    M = oracle.dense_affinity(n, pcol, irow, val, 1.0)
    we, Ve = np.linalg.eigh(M)
    assert np.allclose(w, we[::-1][:4], rtol=1e-10, atol=1e-10)
    assert np.all(res < 1e-8)


def test_oracle_entropic_sigmas_reach_perplexity(oracle):
    """Entropic sigmas: the normalised exp(-d^2/2s^2) over each landmark's
    k-sigma sorted distances has perplexity K (to the 1e-10 root tolerance)."""
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.normal(size=(300, 2)), rng.normal(size=(300, 2)) + 4])
    d, i = oracle.knn_data(x, None, 12)
    n, pc, ir, v = oracle.sysparse(d, i)
    K, ka = 5.0, 10
    sig = oracle.auto_sigmas(n, pc, ir, v, ka, perplexity=K)
    lists = [[] for _ in range(n)]
    for c in range(n):
        for p in range(pc[c], pc[c + 1]):
            lists[c].append(v[p])
            lists[ir[p]].append(v[p])
    for j in range(n):
        a = np.sort(np.array(lists[j][:ka]))
        p = np.exp(-a ** 2 / (2 * sig[j] ** 2))
        p /= p.sum()
        assert abs(-(p * np.log(p)).sum() - np.log(K)) < 1e-8
    # the k-sigma mean is the plain mean of the first ka (by neighbour index), trimmed before sorting
    mean = oracle.auto_sigmas(n, pc, ir, v, ka)
    assert np.allclose(mean, [np.sum(np.sort(lists[j][:ka])) / ka for j in range(n)], rtol=0, atol=1e-15)


def _xtc_frames_end(b):
    """Byte offset where a header walk of an .xtc file ends."""
    import struct

    o = 0
    while o + 56 <= len(b):
        na = struct.unpack(">i", b[o + 4:o + 8])[0]
        if na <= 9:
            o += 56 + 12 * na
        else:
            nb = struct.unpack(">i", b[o + 88:o + 92])[0]
            o += 92 + (nb + 3) // 4 * 4
    return o


def test_oracle_xtc_trp_cage(oracle):
    """The example trajectory decodes to 1000 frames of 60 backbone atoms
    (the topology's count); every N-CA, CA-C and C-N bond of every frame is
    a physical length, and the frames use up the whole file."""
    path = os.path.join(os.path.dirname(__file__), "golden", "trp-cage.xtc")
    b = open(path, "rb").read()
    xyz, steps, times = oracle.xtc_read(b)
    assert xyz.shape == (1000, 60, 3)
    pdb = open(os.path.join(os.path.dirname(__file__), "golden", "trp-cage.pdb")).read().splitlines()
    names = [ln[12:16].strip() for ln in pdb if ln.startswith("ATOM")]
    assert len(names) == 60 and names[:3] == ["N", "CA", "C"]
    assert np.all(np.diff(steps) > 0) and np.all(np.diff(times) > 0)
    bond = np.linalg.norm(xyz[:, 1:] - xyz[:, :-1], axis=2)
    for t, (lo, hi) in enumerate(((0.13, 0.165), (0.135, 0.175), (0.12, 0.15))):  # N-CA, CA-C, C-N
        assert lo < bond[:, t::3].min() and bond[:, t::3].max() < hi
    assert _xtc_frames_end(b) == len(b)


def test_oracle_xtc_synthetic_paths(oracle):
    import xtc_synth as X

    # raw frames (<= 9 atoms)
    q = X.walk(7, 1)
    f = X.encode_frame(q, prec=1000.0, step=5)
    xyz, steps, _ = oracle.xtc_read(f + f)
    assert xyz.shape == (2, 7, 3) and np.array_equal(xyz[0], (q / 1000.0).astype(np.float32))
    # no runs, ranges above 2^24 (fixed-width fields)
    q = X.walk(40, 2, step=3)
    q[5] += 30_000_000
    xyz, _, _ = oracle.xtc_read(X.encode_frame(q, prec=1e6))
    inv = np.float32(1.0 / 1e6)
    assert np.array_equal(xyz[0], q.astype(np.int32).astype(np.float32) * inv)
    # runs, small-index changes, a run reused through a clear flag
    q = X.walk(60, 3)
    groups = [(2, 0, True), (2, 0, False), (0, 0, True), (3, 1, True), (1, -1, True), (5, 0, True),
              (5, 0, False), (0, -1, True), (4, 0, True)]
    groups += [(0, 0, True)] * (60 - sum(g[0] + 1 for g in groups))
    xyz, _, _ = oracle.xtc_read(X.encode_frame(q, prec=1000.0, groups=groups, smallidx=12))
    assert np.array_equal(xyz[0], q.astype(np.int32).astype(np.float32) * np.float32(1.0 / 1000.0))


def test_sparse_distance_oracle_matches_dense(oracle):
    """euclidean_distance_sparse restated: on sorted, repeat-free indices it
    equals the dense Euclidean distance (to rounding; the orders differ)."""
    rng = np.random.default_rng(0)
    vecs = []
    for _ in range(60):
        m = rng.integers(0, 25)
        ii = np.sort(rng.choice(120, m, replace=False))
        vecs.append((ii, rng.normal(size=m)))
    dense = np.zeros((60, 120))
    for r, (ii, vv) in enumerate(vecs):
        dense[r, ii] = vv
    d, i = oracle.knn_data_sparse(oracle.csr(vecs), None, 6)
    full = np.sqrt(((dense[:, None, :] - dense[None, :, :]) ** 2).sum(-1))
    ref = np.take_along_axis(full, i, axis=1)
    assert np.allclose(d, ref, rtol=1e-13, atol=1e-13)
    assert np.allclose(d, np.sort(full, axis=1)[:, 1:7], rtol=1e-13, atol=1e-13)


def test_contact_profile_oracle(oracle):
    rng = np.random.default_rng(1)
    x = rng.uniform(0, 2.5, size=(5, 40, 3)).astype(np.float32)
    g1, g2 = np.arange(10), np.arange(20, 40)
    off, idx = oracle.contact_profile(x, g1, g2, 7.5)
    for f in range(5):
        dd = np.sqrt(((x[f, g1][:, None, :] - x[f, g2][None, :, :]) ** 2).sum(-1).astype(np.float64)) * 10.0
        want = np.flatnonzero((dd < 7.5).reshape(-1))
        assert np.array_equal(idx[off[f]:off[f + 1]], want)
